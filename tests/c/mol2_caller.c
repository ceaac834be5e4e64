/*
 * Calls the reference's libmol2-typed entry points one at a time (through
 * include/compat/ and libfmftsaxs_gb300/mol2/sxs_mol2.c), for the tests:
 *
 *   mol2_caller ff MAPPING_PRM ATOMPRM PDB OUT
 *       per atom "vacuum_ff dummy_ff type" from default_ff_table + get_ff +
 *       atom2ff_type, then a last line with mol_atom_group_average_radius
 *       (src/form_factor_table.c:138-188, 294-339; src/saxs_utils.c:19-28)
 *   mol2_caller expand MAPPING_PRM ATOMPRM PDB OUT L QNUM WATER
 *       atom_grp2spf of the molecule as read (no centring): a line "L qnum rm",
 *       then per q and lm "V.re V.im D.re D.im W.re W.im" at full precision
 *       (src/pdb2spf.c:154-175; GPU)
 *   mol2_caller ft2euler FT RM EULER RX RY RZ
 *       sxs_ft_file2euler_file with ref_lig = (RX, RY, RZ) (src/index.c:77-121)
 */
#include "common.h"

#include "fftsaxs.h"
#include "index.h"

#include "mol2/atom_group.h"
#include "mol2/pdb.h"
#include "mol2/prms.h"
#include "mol2/vector.h"

static struct mol_atom_group *molecule(const char *prm_path, const char *pdb_path)
{
	struct mol_prms *prms = mol_prms_read(prm_path);
	struct mol_atom_group *ag = mol_read_pdb(pdb_path);
	mol_atom_group_add_prms(ag, prms);
	mol_prms_free(prms);
	return ag;
}

int main(int argc, char *argv[])
{
	if (argc >= 6 && !strcmp(argv[1], "ff")) {
		struct saxs_form_factor_table *t = default_ff_table(argv[2]);
		struct mol_atom_group *ag = molecule(argv[3], argv[4]);
		FILE *out = fopen(argv[5], "w");
		CHECK_PTR(out);
		for (size_t i = 0; i < ag->natoms; i++) {
			const struct saxs_form_factor *ff = get_ff(t, ag, i);
			CHECK_PTR(ff);
			fprintf(out, "%.17g %.17g %d\n", ff->vacuum_ff, ff->dummy_ff, (int)atom2ff_type(t, ag, i));
		}
		fprintf(out, "%.17g %.17g\n", mol_atom_group_average_radius(ag), t->factors[s_OH2].zero_ff);
		fclose(out);
		mol_atom_group_free(ag);
		ff_table_destroy(t);
		return 0;
	}
	if (argc >= 9 && !strcmp(argv[1], "expand")) {
		struct saxs_form_factor_table *t = default_ff_table(argv[2]);
		struct mol_atom_group *ag = molecule(argv[3], argv[4]);
		int L = atoi(argv[6]), qnum = atoi(argv[7]), water = atoi(argv[8]);
		double *qvals = sxs_mkarray(0.0, QMAX, qnum);
		struct sxs_spf_full *spf = atom_grp2spf(ag, t, qvals, qnum, L, water);
		FILE *out = fopen(argv[5], "w");
		CHECK_PTR(out);
		fprintf(out, "%d %d %.17g\n", spf->L, spf->qnum, spf->rm);
		for (int q = 0; q < qnum; q++)
			for (int i = 0; i < (L + 1) * (L + 1); i++)
				fprintf(out, "%.17g %.17g %.17g %.17g %.17g %.17g\n", spf->V[q]->re[i], spf->V[q]->im[i],
				        spf->D[q]->re[i], spf->D[q]->im[i], spf->W[q]->re[i], spf->W[q]->im[i]);
		fclose(out);
		sxs_spf_full_free(spf);
		sxs_myfree(qvals);
		mol_atom_group_free(ag);
		ff_table_destroy(t);
		return 0;
	}
	if (argc >= 8 && !strcmp(argv[1], "ft2euler")) {
		struct mol_vector3 ref = {atof(argv[5]), atof(argv[6]), atof(argv[7])};
		sxs_ft_file2euler_file(argv[4], argv[2], argv[3], &ref);
		return 0;
	}
	fprintf(stderr, "usage: see the comment at the top of mol2_caller.c\n");
	return 2;
}
