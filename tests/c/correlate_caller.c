/*
 * A scoring program written the way the reference's tools/correlate.c is
 * (:74-105 form factors, molecules and their expansions; :125-135 the
 * experiment and fit parameters; :264-281 scoring) with the Euler-file
 * reading of tests/saxs_test.c:243-320, using only the reference's API and
 * libmol2.  It includes the reference's header names, which
 * include/compat/ provides, and links against libfmftsaxs_gb300.so plus
 * libfmftsaxs_gb300/mol2/sxs_mol2.c; in the tests libmol2 is the stand-in
 * of tests/c/mol2_stub.c.
 *
 * Usage: correlate_caller MAPPING_PRM ATOMPRM REC LIG SAXS_PROFILE EULER OUTPUT
 *                         L QNUM QMAX Z_BEG Z_END Z_STEP
 * Output: "id chi c1 c2" (17 significant digits) per Euler line whose z is
 * on the translation grid, in file order.
 */
#include "common.h"

#include "fftsaxs.h"
#include "index.h"

#include "mol2/atom_group.h"
#include "mol2/pdb.h"
#include "mol2/prms.h"
#include "mol2/vector.h"

int main(int argc, char *argv[])
{
	if (argc != 14) {
		fprintf(stderr, "Usage: %s MAPPING_PRM ATOMPRM REC LIG SAXS_PROFILE EULER OUTPUT L QNUM QMAX Z_BEG Z_END "
		                "Z_STEP\n", argv[0]);
		exit(EXIT_FAILURE);
	}
	char *map_path = argv[1];
	char *prm_path = argv[2];
	char *rec_path = argv[3];
	char *lig_path = argv[4];
	char *exp_path = argv[5];
	char *eul_path = argv[6];
	char *out_path = argv[7];
	int L = atoi(argv[8]);
	int qnum = atoi(argv[9]);
	double qmax = atof(argv[10]);
	double z_beg = atof(argv[11]);
	double z_end = atof(argv[12]);
	double z_step = atof(argv[13]);
	int nbeta = L + 1;

	double *qvals = sxs_mkarray(0.0, qmax, qnum);
	struct mol_prms *prms = mol_prms_read(prm_path);
	struct saxs_form_factor_table *ff_table = default_ff_table(map_path);

	/* receptor, centred at its centre of extrema */
	struct mol_atom_group *pa1 = mol_read_pdb(rec_path);
	mol_atom_group_add_prms(pa1, prms);
	struct mol_vector3 coe;
	center_of_extrema(&coe, pa1);
	MOL_VEC_MULT_SCALAR(coe, coe, -1.0);
	mol_atom_group_translate(pa1, &coe);
	struct sxs_spf_full *A = atom_grp2spf(pa1, ff_table, qvals, qnum, L, 1);

	/* ligand, centred at its centroid */
	struct mol_atom_group *pa2 = mol_read_pdb(lig_path);
	mol_atom_group_add_prms(pa2, prms);
	struct mol_vector3 com;
	centroid(&com, pa2);
	MOL_VEC_MULT_SCALAR(com, com, -1.0);
	mol_atom_group_translate(pa2, &com);
	struct sxs_spf_full *B = atom_grp2spf(pa2, ff_table, qvals, qnum, L, 1);

	/* experiment and fit parameters */
	struct sxs_profile *exp_profile = sxs_profile_read(exp_path);
	double mean_radius = (A->rm * pa1->natoms + B->rm * pa2->natoms) / (pa1->natoms + pa2->natoms);
	struct sxs_opt_params *params = sxs_opt_params_create(exp_profile, qvals, qnum, mean_radius);
	mol_prms_free(prms);
	free(exp_profile->qvals);
	sxs_profile_free(exp_profile);

	/* translation grid */
	int znum_total = (int)round((z_end - z_beg) / z_step) + 1;
	double *zvals = calloc(znum_total, sizeof(double));
	int znum = 0;
	for (double zval = z_beg; zval < (z_end + 0.001); zval += z_step) zvals[znum++] = zval;

	/* Euler file -> grid indices (no wrap of the angle digits) */
	FILE *euler_file = fopen(eul_path, "r");
	CHECK_PTR(euler_file);
	int ft_id, ft_num = 0, nread;
	double z, line[5];
	while ((nread = fscanf(euler_file, "%d %lf %lf %lf %lf %lf %lf", &ft_id, &z, &line[0], &line[1], &line[2],
	                       &line[3], &line[4])) != EOF) {
		if (nread != 7) ERROR_MSG("Wrong Euler file format.");
		for (int j = 0; j < znum; j++)
			if (zvals[j] > z - 0.001 && zvals[j] < z + 0.001) ft_num++;
	}
	rewind(euler_file);
	int *saxs_index = calloc(ft_num, sizeof(int));
	int *ft_index = calloc(ft_num, sizeof(int));
	double *saxs_score = calloc(ft_num, sizeof(double));
	double *c1_list = calloc(ft_num, sizeof(double));
	double *c2_list = calloc(ft_num, sizeof(double));
	double b_step = M_PI / L;
	double a_step = 2.0 * M_PI / (2 * L + 1);
	struct sxs_euler euler;
	int counter = 0;
	while ((nread = fscanf(euler_file, "%d %lf %lf %lf %lf %lf %lf", &ft_id, &euler.z, &euler.b1, &euler.g1,
	                       &euler.a2, &euler.b2, &euler.g2)) != EOF) {
		if (nread != 7) ERROR_MSG("Wrong Euler file format.");
		for (int j = 0; j < znum; j++) {
			if (zvals[j] > euler.z - 0.001 && zvals[j] < euler.z + 0.001) {
				euler.a2 = 2 * M_PI - euler.a2;
				euler.g2 = 2 * M_PI - euler.g2;
				int tmp_id = (int)(round((euler.z - z_beg) / z_step)) * nbeta;
				tmp_id = (tmp_id + (int)round(euler.b1 / b_step)) * nbeta;
				tmp_id = (tmp_id + (int)round(euler.b2 / b_step)) * (2 * L + 1);
				tmp_id = (tmp_id + (int)round(euler.a2 / a_step)) * (2 * L + 1);
				tmp_id = (tmp_id + (int)round(euler.g1 / a_step)) * (2 * L + 1);
				tmp_id = tmp_id + (int)round(euler.g2 / a_step);
				saxs_index[counter] = tmp_id;
				ft_index[counter] = ft_id;
				counter++;
			}
		}
	}
	fclose(euler_file);

	sxs_compute_saxs_scores(saxs_score, c1_list, c2_list, saxs_index, ft_num, A, B, params, qvals, qnum, zvals, znum,
	                        L, 1);

	FILE *out = fopen(out_path, "w");
	CHECK_PTR(out);
	for (int i = 0; i < ft_num; i++)
		fprintf(out, "%d %.17g %.17g %.17g\n", ft_index[i], saxs_score[i], c1_list[i], c2_list[i]);
	fclose(out);

	sxs_myfree(saxs_score);
	sxs_myfree(saxs_index);
	sxs_myfree(ft_index);
	sxs_myfree(c1_list);
	sxs_myfree(c2_list);
	sxs_myfree(zvals);
	sxs_opt_params_free(params);
	sxs_spf_full_free(A);
	sxs_spf_full_free(B);
	mol_atom_group_free(pa1);
	mol_atom_group_free(pa2);
	ff_table_destroy(ff_table);
	sxs_myfree(qvals);
	return 0;
}
