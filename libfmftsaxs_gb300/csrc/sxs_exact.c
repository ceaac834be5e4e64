/*
 * Exact per-pose scoring: the flow of the reference's score_ft_naive tool
 * (tools/score_ft_naive.c:156-212) on the GPU, for cross-checking the grid
 * method on chosen poses.  For each Euler pose (z, beta1, gamma1, alpha2,
 * beta2, gamma2):
 *   receptor atoms -> R(0, beta1, gamma1) x            (active rotation,
 *   ligand atoms   -> R(alpha2, beta2, gamma2) x + (0, 0, z)   src/saxs_utils.c)
 *   joined complex (receptor first) -> minus its centroid
 *   -> A_lm expansion of the complex (the kernels of sxsg_expand)
 *   -> single-molecule cross terms (sxs_spf2cross_terms, src/min_saxs.c:450)
 *   -> L-BFGS-B fit of (c1, c2) without the peak rescale (sxs_lbfgs_fitting,
 *      as sxs_spf2fitted_profile calls it, src/min_saxs.c:496-511).
 * The moves follow libmol2's mol_atom_group_move_in_copy and centroid
 * (absent from the reference tree): x' = m11 x + m12 y + m13 z + t, summed
 * left to right; the centroid is the plain sum over atoms divided by n.
 * Water weights (water form factor x accessible fraction per atom of the
 * joined order) are an input: the tool computes them once, on the unmoved
 * join, and reuses them for every pose.
 */
#define _XOPEN_SOURCE 700
#include <math.h>
#include <stdlib.h>
#include <string.h>

#include "sxs_internal.h"

#define SXS_EXACT_BATCH 128

static void move_atoms(const double *src, int n, const struct mol_matrix3 *r, double tz, double *dst)
{
	for (int i = 0; i < n; i++) {
		double x = src[3 * i], y = src[3 * i + 1], z = src[3 * i + 2];
		dst[3 * i] = r->m11 * x + r->m12 * y + r->m13 * z + 0.0;
		dst[3 * i + 1] = r->m21 * x + r->m22 * y + r->m23 * z + 0.0;
		dst[3 * i + 2] = r->m31 * x + r->m32 * y + r->m33 * z + tz;
	}
}

/* joined, centred coordinates of one pose into out[3 (nrec + nlig)] */
void sxs_exact_pose_coords(const double *rec, int nrec, const double *lig, int nlig, const double *eu6, double *out)
{
	struct mol_matrix3 rr, lr;
	sxs_fill_active_rotation_matrix(&rr, 0.0, eu6[1], eu6[2]);
	sxs_fill_active_rotation_matrix(&lr, eu6[3], eu6[4], eu6[5]);
	move_atoms(rec, nrec, &rr, 0.0, out);
	move_atoms(lig, nlig, &lr, eu6[0], out + 3 * (size_t)nrec);
	int n = nrec + nlig;
	double cx = 0.0, cy = 0.0, cz = 0.0;
	for (int i = 0; i < n; i++) {
		cx += out[3 * i];
		cy += out[3 * i + 1];
		cz += out[3 * i + 2];
	}
	if (n > 0) {
		cx = -(cx / n);
		cy = -(cy / n);
		cz = -(cz / n);
	}
	for (int i = 0; i < n; i++) {
		out[3 * i] += cx;
		out[3 * i + 1] += cy;
		out[3 * i + 2] += cz;
	}
}

int sxsg_score_exact(const double *rec_xyz, int nrec, const double *lig_xyz, int nlig, const double *vac,
                     const double *dum, const double *water_w, const double *euler, int64_t n, const double *q, int Q,
                     int L, const double *a, double mult, double *chi, double *c1, double *c2, double *cross)
{
	if (nrec < 0 || nlig < 0 || nrec + nlig <= 0 || !rec_xyz || !lig_xyz || !vac || !dum || !euler || n < 0 ||
	    !q || Q <= 0 || !a)
		return sxs_fail(-2, "sxsg_score_exact: bad arguments");
	if (n == 0) return 0;
	const sxs_ltables *lt;
	int rc = sxs_ltables_get(L, &lt);
	if (rc) return rc;
	cudaStream_t s = sxs_default_stream();
	int na = nrec + nlig, K = L + 1;
	int B = n < SXS_EXACT_BATCH ? (int)n : SXS_EXACT_BATCH;
	size_t spf_n = (size_t)3 * Q * K * K * 2;
	double *h_xyz = malloc(sizeof(double) * 3 * na * (size_t)B);
	double *wf = calloc(na, sizeof(double));
	if (!h_xyz || !wf) {
		free(h_xyz); free(wf);
		return sxs_fail(-5, "out of host memory");
	}
	if (water_w) memcpy(wf, water_w, sizeof(double) * na);
	double *d_xyz = NULL, *d_vac = NULL, *d_dum = NULL, *d_wf = NULL, *d_q = NULL, *d_a = NULL, *d_rad = NULL;
	double *d_spf = NULL, *d_cross = NULL, *d_ct = NULL, *d_chi = NULL, *d_c1 = NULL, *d_c2 = NULL;
	double2 *d_ylm = NULL;
	cudaError_t e = cudaSuccess;
	if (!e) e = cudaMalloc((void **)&d_xyz, sizeof(double) * 3 * na * (size_t)B);
	if (!e) e = cudaMalloc((void **)&d_vac, sizeof(double) * na);
	if (!e) e = cudaMalloc((void **)&d_dum, sizeof(double) * na);
	if (!e) e = cudaMalloc((void **)&d_wf, sizeof(double) * na);
	if (!e) e = cudaMalloc((void **)&d_q, sizeof(double) * Q);
	if (!e) e = cudaMalloc((void **)&d_a, sizeof(double) * 6 * Q);
	if (!e) e = cudaMalloc((void **)&d_rad, sxsk_expand_ws_rad(na));
	if (!e) e = cudaMalloc((void **)&d_ylm, sxsk_expand_ws_ylm(na, L));
	if (!e) e = cudaMalloc((void **)&d_spf, sizeof(double) * spf_n * B);
	if (!e) e = cudaMalloc((void **)&d_cross, sizeof(double) * 6 * Q * (size_t)B);
	if (!e) e = cudaMalloc((void **)&d_ct, sizeof(double) * 6 * Q * (size_t)B);
	if (!e) e = cudaMalloc((void **)&d_chi, sizeof(double) * B);
	if (!e) e = cudaMalloc((void **)&d_c1, sizeof(double) * B);
	if (!e) e = cudaMalloc((void **)&d_c2, sizeof(double) * B);
	if (!e) e = cudaMemcpyAsync(d_vac, vac, sizeof(double) * na, cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(d_dum, dum, sizeof(double) * na, cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(d_wf, wf, sizeof(double) * na, cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(d_q, q, sizeof(double) * Q, cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(d_a, a, sizeof(double) * 6 * Q, cudaMemcpyHostToDevice, s);
	for (int64_t p0 = 0; p0 < n && !e; p0 += B) {
		int nb = (int)(n - p0 < B ? n - p0 : B);
		for (int k = 0; k < nb; k++)
			sxs_exact_pose_coords(rec_xyz, nrec, lig_xyz, nlig, euler + 6 * (p0 + k), h_xyz + 3 * (size_t)na * k);
		e = cudaMemcpyAsync(d_xyz, h_xyz, sizeof(double) * 3 * na * (size_t)nb, cudaMemcpyHostToDevice, s);
		for (int k = 0; k < nb && !e; k++)
			e = (cudaError_t)sxsk_expand(d_xyz + 3 * (size_t)na * k, d_vac, d_dum, d_wf, na, d_q, Q, L, lt->d_ynorm,
			                             d_ylm, d_rad, d_spf + spf_n * k, s);
		if (!e) e = (cudaError_t)sxsk_self_cross(d_spf, nb, Q, L, d_cross, s);
		if (!e)
			e = (cudaError_t)sxs_fit_lbfgsb_launch(d_cross, 0, d_ct, nb, Q, d_q, d_a, mult, 1.0, 0, d_chi, d_c1, d_c2, NULL,
			                                       NULL, s);
		sxs_count_launches(sxsk_expand_launches() * nb + 3);
		if (!e && chi) e = cudaMemcpyAsync(chi + p0, d_chi, sizeof(double) * nb, cudaMemcpyDeviceToHost, s);
		if (!e && c1) e = cudaMemcpyAsync(c1 + p0, d_c1, sizeof(double) * nb, cudaMemcpyDeviceToHost, s);
		if (!e && c2) e = cudaMemcpyAsync(c2 + p0, d_c2, sizeof(double) * nb, cudaMemcpyDeviceToHost, s);
		if (!e && cross)
			e = cudaMemcpyAsync(cross + 6 * Q * p0, d_cross, sizeof(double) * 6 * Q * (size_t)nb,
			                    cudaMemcpyDeviceToHost, s);
		if (!e) e = cudaStreamSynchronize(s);
	}
	cudaFree(d_xyz); cudaFree(d_vac); cudaFree(d_dum); cudaFree(d_wf); cudaFree(d_q); cudaFree(d_a);
	cudaFree(d_rad); cudaFree(d_ylm); cudaFree(d_spf); cudaFree(d_cross); cudaFree(d_ct);
	cudaFree(d_chi); cudaFree(d_c1); cudaFree(d_c2);
	free(h_xyz); free(wf);
	if (e) return sxs_cuda_fail(e, "sxsg_score_exact");
	return 0;
}

/* Accessible fraction of every atom (Shrake-Rupley on the sphere points
 * sph[npts][3], or a golden spiral of npts points when sph is NULL): the
 * W-channel weights of the expansion, computed on the device. */
int sxsg_sasa(const double *xyz, const double *radius, int natoms, double probe, const double *sph, int npts,
              double *frac)
{
	if (natoms < 0 || (natoms > 0 && (!xyz || !radius || !frac)) || npts <= 0 || npts > 1024)
		return sxs_fail(-2, "sxsg_sasa: bad arguments (1 <= npts <= 1024)");
	if (natoms == 0) return 0;
	int rc = sxs_ensure_init();
	if (rc) return rc;
	cudaStream_t s = sxs_default_stream();
	double *h_sph = NULL;
	if (!sph) {
		h_sph = malloc(sizeof(double) * 3 * npts);
		if (!h_sph) return sxs_fail(-5, "out of host memory");
		for (int k = 0; k < npts; k++) {
			double kk = k + 0.5;
			double phi = acos(1.0 - 2.0 * kk / npts);
			double th = SXS_PI_FULL * (1.0 + sqrt(5.0)) * kk;
			h_sph[3 * k] = cos(th) * sin(phi);
			h_sph[3 * k + 1] = sin(th) * sin(phi);
			h_sph[3 * k + 2] = cos(phi);
		}
		sph = h_sph;
	}
	double *d_xyz = NULL, *d_rad = NULL, *d_sph = NULL, *d_f = NULL;
	cudaError_t e = cudaMalloc((void **)&d_xyz, sizeof(double) * 3 * natoms);
	if (!e) e = cudaMalloc((void **)&d_rad, sizeof(double) * natoms);
	if (!e) e = cudaMalloc((void **)&d_sph, sizeof(double) * 3 * npts);
	if (!e) e = cudaMalloc((void **)&d_f, sizeof(double) * natoms);
	if (!e) e = cudaMemcpyAsync(d_xyz, xyz, sizeof(double) * 3 * natoms, cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(d_rad, radius, sizeof(double) * natoms, cudaMemcpyHostToDevice, s);
	if (!e) e = cudaMemcpyAsync(d_sph, sph, sizeof(double) * 3 * npts, cudaMemcpyHostToDevice, s);
	if (!e) {
		e = (cudaError_t)sxsk_sasa(d_xyz, d_rad, natoms, probe, d_sph, npts, d_f, s);
		sxs_count_launches(1);
	}
	if (!e) e = cudaMemcpyAsync(frac, d_f, sizeof(double) * natoms, cudaMemcpyDeviceToHost, s);
	if (!e) e = cudaStreamSynchronize(s);
	cudaFree(d_xyz); cudaFree(d_rad); cudaFree(d_sph); cudaFree(d_f);
	free(h_sph);
	if (e) return sxs_cuda_fail(e, "sxsg_sasa");
	return 0;
}
