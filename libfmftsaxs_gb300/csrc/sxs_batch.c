/*
 * Batches of dimers: many mixed-precision plans (each one dimer with its own
 * L, q grid, experiment, pose list and fit grid) scored by one CUDA graph.
 *
 * Work items.  Every stage of a plan run is a grid of independent blocks:
 * rotation blocks (table, q tile, beta, m), translation blocks (chunk, q
 * tile, slice group, m) per column class NB, per-pose blocks (chunk, q tile,
 * 32 poses) and fit groups (dimer, group of poses).  The batch lists those
 * blocks of all dimers as (job, ...) items: jobs by estimated cost, largest
 * first, the items of a job in the single-dimer kernel's block order (its
 * L2 reuse between neighbouring blocks).  Each list runs as one launch:
 * persistent (SMs x resident blocks taking items through an atomic counter,
 * SXSG_BATCH_PERSISTENT) or one block per item.  An item runs the
 * single-dimer kernel's own block code, so every output equals a
 * sxsg_plan_run of its plan bit for bit.
 *
 * Phases.  The translated table of a dimer is cut into chunks of whole
 * slices (as a plan run does); chunks of all dimers are packed first-fit,
 * largest first, into phases whose chunks fit one shared device arena.  A
 * phase is the translation of its chunks (a stream per column class, the
 * classes on parallel branches of the graph) followed by their per-pose
 * work.  By default those are the single-dimer launches of each chunk (they
 * measured faster than work-item launches of the same blocks); with
 * SXSG_BATCH_ITEMS they are work-item launches over all the phase's chunks.
 * The rotations and the fit are always work-item launches.
 *
 * Graph.  Zeroing the item counters, the per-z tables of every dimer (two
 * high-priority branches, so that their FP64 blocks run beside the rotation
 * blocks), the rotation launches (one per gamma group size), the phases and
 * the fit launch are captured once at sxsg_batch_create; a run is one
 * cudaGraphLaunch.  Stage times come from event nodes in the graph.
 */
#include <stdlib.h>
#include <string.h>

#include "sxs_internal.h"

#define SXSB_BR 8        /* branch streams of the capture */
#define SXSB_ALIGN 256

typedef struct {
	double cost;
	int64_t seq;
	int4 w;
} bitem;

typedef struct {
	int plan;
	int64_t s0, s1;          /* slices */
	int64_t c0, c1;          /* combos */
	size_t bytes;
	int phase;
	size_t off;              /* in the arena */
} bpiece;

typedef struct {
	int kind;                /* 0 rotation, 1 translation, 2 per-pose, 3 fit, 4 fused translation,
	                          * 5 sums over m of the fused path */
	int arg;                 /* G or NB */
	int phase;
	int nitems, njobs;
	size_t jobs_off, items_off;
	int ctr;                 /* counter slot */
} blaunch;

struct sxsg_batch {
	int n, fit_mode;
	sxsg_plan **plans;
	sxs_plan_view *v;
	int flags;
	cudaStream_t s, ps, br[SXSB_BR];   /* origin (tables, fit), pose lane, translation lanes */
	cudaEvent_t fork, join[SXSB_BR], evpose[2];
	cudaEvent_t ev[4];       /* graph event nodes: start, tables done, phases done, end */
	cudaGraph_t graph;
	cudaGraphExec_t exec;
	void *d_buf, *d_arena;
	size_t arena;
	size_t fit_smem;
	int nphase, nlaunch, nkern;
	int64_t nitems, nposes;
	double ms[4];
};

static int cmp_item(const void *a, const void *b)
{
	const bitem *x = a, *y = b;
	if (x->cost != y->cost) return x->cost > y->cost ? -1 : 1;
	return x->seq < y->seq ? -1 : (x->seq > y->seq);
}

static int cmp_piece(const void *a, const void *b)
{
	const bpiece *x = a, *y = b;
	if (x->bytes != y->bytes) return x->bytes > y->bytes ? -1 : 1;
	if (x->plan != y->plan) return x->plan < y->plan ? -1 : 1;
	return x->s0 < y->s0 ? -1 : (x->s0 > y->s0);
}

/* growable host arrays */
typedef struct {
	void *p;
	size_t n, cap, elem;
} bvec;

static void *bv_push(bvec *v)
{
	if (v->n == v->cap) {
		size_t nc = v->cap ? 2 * v->cap : 256;
		void *q = realloc(v->p, nc * v->elem);
		if (!q) return NULL;
		v->p = q;
		v->cap = nc;
	}
	return (char *)v->p + v->elem * v->n++;
}

static size_t al(size_t x) { return (x + SXSB_ALIGN - 1) & ~(size_t)(SXSB_ALIGN - 1); }

/* bytes of one combo's translated rows */
static size_t combo_bytes(const sxs_plan_view *v) { return (size_t)v->NP * 3 * SXS_QT * v->NT * sizeof(float2); }

void sxsg_batch_destroy(sxsg_batch *b)
{
	if (!b) return;
	if (b->s) cudaStreamSynchronize(b->s);
	if (b->exec) cudaGraphExecDestroy(b->exec);
	if (b->graph) cudaGraphDestroy(b->graph);
	if (b->d_buf) cudaFree(b->d_buf);
	if (b->d_arena) {
		cudaFreeAsync(b->d_arena, b->s);
		cudaStreamSynchronize(b->s);
	}
	for (int i = 0; i < SXSB_BR; i++) {
		if (b->br[i]) cudaStreamDestroy(b->br[i]);
		if (b->join[i]) cudaEventDestroy(b->join[i]);
	}
	for (int i = 0; i < 4; i++)
		if (b->ev[i]) cudaEventDestroy(b->ev[i]);
	for (int i = 0; i < 2; i++)
		if (b->evpose[i]) cudaEventDestroy(b->evpose[i]);
	if (b->fork) cudaEventDestroy(b->fork);
	if (b->ps) cudaStreamDestroy(b->ps);
	if (b->s) cudaStreamDestroy(b->s);
	free(b->plans);
	free(b->v);
	free(b);
}

/* Host side of the work lists: jobs and items of every launch in one
 * staging buffer (offsets into the device copy), launches in graph order. */
typedef struct {
	char *h;
	size_t used, cap;
	bvec launches;
} bstage;

static size_t st_put(bstage *st, const void *src, size_t bytes)
{
	size_t off = al(st->used);
	if (off + bytes > st->cap) {
		size_t nc = st->cap ? st->cap : 1 << 20;
		while (nc < off + bytes) nc *= 2;
		char *q = realloc(st->h, nc);
		if (!q) return (size_t)-1;
		st->h = q;
		st->cap = nc;
	}
	if (bytes) memcpy(st->h + off, src, bytes);
	st->used = off + bytes;
	return off;
}

/* sorts items (largest cost first), stores the jobs and items, appends the
 * launch */
static int st_launch(bstage *st, int kind, int arg, int phase, const void *jobs, size_t jbytes, int njobs,
                     bvec *items, int pair)
{
	/* a launch over work items, or (no items) one launch per job */
	if (njobs == 0 || (items->n == 0 && kind != 1 && kind != 2 && kind != 4 && kind != 5)) return 0;
	if (items->n > INT32_MAX) return sxs_fail(-2, "sxsg_batch_create: too many work items in one launch");
	qsort(items->p, items->n, sizeof(bitem), cmp_item);
	size_t ib = items->n * (pair ? sizeof(int2) : sizeof(int4));
	char *tmp = malloc(ib > 0 ? ib : 1);
	if (!tmp) return sxs_fail(-5, "out of host memory");
	const bitem *it = items->p;
	for (size_t i = 0; i < items->n; i++) {
		if (pair) {
			int2 w = {it[i].w.x, it[i].w.y};
			memcpy(tmp + i * sizeof(int2), &w, sizeof(w));
		} else {
			memcpy(tmp + i * sizeof(int4), &it[i].w, sizeof(int4));
		}
	}
	blaunch *L = bv_push(&st->launches);
	if (!L) {
		free(tmp);
		return sxs_fail(-5, "out of host memory");
	}
	L->kind = kind;
	L->arg = arg;
	L->phase = phase;
	L->nitems = (int)items->n;
	L->njobs = njobs;
	L->jobs_off = st_put(st, jobs, jbytes);
	L->items_off = st_put(st, tmp, ib);
	L->ctr = (int)st->launches.n - 1;
	free(tmp);
	items->n = 0;
	if (L->jobs_off == (size_t)-1 || L->items_off == (size_t)-1) return sxs_fail(-5, "out of host memory");
	return 0;
}

static int add_item(bvec *items, double cost, int x, int y, int z, int w)
{
	bitem *it = bv_push(items);
	if (!it) return sxs_fail(-5, "out of host memory");
	it->cost = cost;
	it->seq = (int64_t)items->n;
	it->w.x = x;
	it->w.y = y;
	it->w.z = z;
	it->w.w = w;
	return 0;
}

/* Items [i0, n) are one job's, added in the single-dimer kernel's block
 * order; they all get the job's total cost, so that a launch takes the jobs
 * largest first and the blocks of each job in that order (neighbouring
 * blocks share table rows in L2 as in the single-dimer launch). */
static void job_cost(bvec *items, size_t i0)
{
	bitem *it = items->p;
	double tot = 0;
	for (size_t i = i0; i < items->n; i++) tot += it[i].cost;
	for (size_t i = i0; i < items->n; i++) it[i].cost = tot;
}

/* rotation launches: one per gamma group size, items (table, t, b, m) */
static int build_rotations(sxsg_batch *b, bstage *st)
{
	static const int gs[6] = {2, 4, 6, 8, 12, 16};
	bvec items = {NULL, 0, 0, sizeof(bitem)};
	int rc = 0;
	sxsk_rot_job *jobs = malloc(sizeof(sxsk_rot_job) * 2 * (size_t)b->n);
	if (!jobs) return sxs_fail(-5, "out of host memory");
	for (int gi = 0; gi < 6 && !rc; gi++) {
		int G = gs[gi], nj = 0, twmax = 0;
		for (int i = 0; i < b->n && !rc; i++) {
			const sxs_plan_view *v = &b->v[i];
			if (sxsk_rotate_group(v->L, v->rot_gamma) != G) continue;
			int K = v->L + 1, N = 2 * v->L + 1;
			int tw = N + (G - 1) * v->L;
			if (tw > twmax) twmax = tw;
			for (int tab = 0; tab < 2; tab++) {
				sxsk_rot_job *j = &jobs[nj];
				memset(j, 0, sizeof(*j));
				j->spf_t = tab ? v->Bt : v->At;
				j->dtab = v->dtabf;
				j->tw = v->tw;
				j->out = tab ? v->U : v->P;
				j->Q = v->Q;
				j->L = v->L;
				j->conj = tab;
				size_t i0 = items.n;
				for (int t = 0; t < v->NT && !rc; t++)
					for (int bb = 0; bb < K && !rc; bb++)
						for (int m = 0; m < K && !rc; m++) {
							/* multiply-adds of the block: sum over l >= m of l */
							double cost = 0.5 * ((double)v->L * (v->L + 1) - (double)m * (m - 1)) + (K - m);
							rc = add_item(&items, cost, nj, t, bb, m);
						}
				job_cost(&items, i0);
				nj++;
			}
		}
		if (!rc) rc = st_launch(st, 0, G | (twmax << 8), -1, jobs, sizeof(sxsk_rot_job) * nj, nj, &items, 0);
	}
	free(jobs);
	free(items.p);
	return rc;
}

/* chunks of every dimer's translated table, packed into phases */
/* First fit: item k (of bytes[k] <= cap, in the given order) goes to the
 * first phase with room, at offset off[k] there; returns the number of
 * phases and in *used the fullest phase's bytes.  The batch passes its
 * chunks largest first. */
int sxs_pack_first_fit(const size_t *bytes, size_t n, size_t cap, int *phase, size_t *off, size_t *used)
{
	size_t *fill = calloc(n > 0 ? n : 1, sizeof(size_t));
	int nphase = 0;
	if (!fill) return -1;
	for (size_t k = 0; k < n; k++) {
		int ph = 0;
		while (ph < nphase && fill[ph] + bytes[k] > cap) ph++;
		if (ph == nphase) nphase++;
		phase[k] = ph;
		off[k] = fill[ph];
		fill[ph] += bytes[k];
	}
	size_t u = 0;
	for (int ph = 0; ph < nphase; ph++) u = fill[ph] > u ? fill[ph] : u;
	free(fill);
	*used = u;
	return nphase;
}

/* device bytes of a piece's slices [s0, s1): its translated rows, or on the
 * fused path its poses' per-m sums */
static size_t piece_bytes(const sxs_plan_view *v, int64_t s0, int64_t s1)
{
	int64_t c0 = v->h_slices[2 * s0], c1 = v->h_slices[2 * (s1 - 1)] + v->h_slices[2 * (s1 - 1) + 1];
	if (v->fused) return al(sizeof(float) * sxsk_fused_part_floats(v->L, v->Q) * (size_t)(v->h_cstart[c1] - v->h_cstart[c0]));
	return al(combo_bytes(v) * (size_t)(c1 - c0));
}

/* translation items of one job for column class NB: (job, t, slice group, m)
 * in the single-dimer block order, costed by combos x n^2 */
static int tr_items(bvec *items, int j, const sxs_plan_view *v, const int32_t *hs, int nslice, int sb, int NB)
{
	int K = v->L + 1, rc = 0;
	int m_hi = K - (NB - 3), m_lo = K - NB;
	if (m_hi > v->L) m_hi = v->L;
	if (m_lo < 0) m_lo = 0;
	int ng = (nslice + sb - 1) / sb;
	size_t i0 = items->n;
	for (int tt = 0; tt < v->NT && !rc; tt++)
		for (int g = 0; g < ng && !rc; g++) {
			int sa = g * sb, sz = sa + sb < nslice ? sa + sb : nslice;
			double nc = (double)(hs[2 * (sz - 1)] + hs[2 * (sz - 1) + 1] - hs[2 * sa]);
			for (int m = m_lo; m <= m_hi && !rc; m++) rc = add_item(items, nc * (K - m) * (K - m), j, tt, g, m);
		}
	job_cost(items, i0);
	return rc;
}

static int build_phases(sxsg_batch *b, bstage *st, size_t arena_req)
{
	bvec pieces = {NULL, 0, 0, sizeof(bpiece)};
	int rc = 0;
	size_t total = 0, largest_slice = 0;
	for (int i = 0; i < b->n; i++) {
		const sxs_plan_view *v = &b->v[i];
		if (v->nslice <= 0) continue;
		for (int64_t k = 0; k < v->nslice; k++) {
			size_t sl = piece_bytes(v, k, k + 1);
			if (sl > largest_slice) largest_slice = sl;
		}
		total += piece_bytes(v, 0, v->nslice);
	}
	size_t fr = 0, tot = 0;
	cudaMemGetInfo(&fr, &tot);
	int halves = (b->flags & SXSG_BATCH_OVERLAP) ? 2 : 1;
	size_t arena = arena_req ? arena_req : fr / 2;
	if (arena > total * halves) arena = total * halves;
	arena = arena / halves & ~(size_t)(SXSB_ALIGN - 1);   /* one phase's share */
	if (total > 0 && arena < largest_slice) {
		if (arena_req) return sxs_fail(-2, "sxsg_batch_create: arena of %zu bytes below one slice (%zu)", arena_req,
		                               largest_slice);
		return sxs_fail(-5, "sxsg_batch_create: free device memory below one slice of a translated table");
	}
	/* pieces: runs of whole slices that fit the arena share */
	for (int i = 0; i < b->n && !rc; i++) {
		const sxs_plan_view *v = &b->v[i];
		int64_t s0 = 0;
		while (s0 < v->nslice && !rc) {
			int64_t s1 = s0 + 1;
			while (s1 < v->nslice && piece_bytes(v, s0, s1 + 1) <= arena) s1++;
			bpiece *p = bv_push(&pieces);
			if (!p) {
				rc = sxs_fail(-5, "out of host memory");
				break;
			}
			p->plan = i;
			p->s0 = s0;
			p->s1 = s1;
			p->c0 = v->h_slices[2 * s0];
			p->c1 = v->h_slices[2 * (s1 - 1)] + v->h_slices[2 * (s1 - 1) + 1];
			p->bytes = piece_bytes(v, s0, s1);
			p->phase = -1;
			s0 = s1;
		}
	}
	if (rc) {
		free(pieces.p);
		return rc;
	}
	bpiece *pc = pieces.p;
	size_t np = pieces.n;
	qsort(pc, np, sizeof(bpiece), cmp_piece);
	/* first fit, largest first */
	size_t *pb = malloc(sizeof(size_t) * (np > 0 ? np : 1)), *po = malloc(sizeof(size_t) * (np > 0 ? np : 1));
	int *pp = malloc(sizeof(int) * (np > 0 ? np : 1));
	if (!pb || !po || !pp) {
		free(pb); free(po); free(pp); free(pieces.p);
		return sxs_fail(-5, "out of host memory");
	}
	for (size_t k = 0; k < np; k++) pb[k] = pc[k].bytes;
	size_t used = 0;
	int nphase = sxs_pack_first_fit(pb, np, arena, pp, po, &used);
	if (nphase < 0) {
		free(pb); free(po); free(pp); free(pieces.p);
		return sxs_fail(-5, "out of host memory");
	}
	for (size_t k = 0; k < np; k++) {
		pc[k].phase = pp[k];
		pc[k].off = po[k];
	}
	free(pb); free(po); free(pp);
	/* phase k uses arena half k mod halves */
	for (size_t k = 0; k < np; k++) pc[k].off += (size_t)(pc[k].phase % halves) * used;
	if (nphase < 2) halves = 1;
	used *= (size_t)halves;
	b->nphase = nphase;
	b->arena = used;
	if (used > 0) {
		/* from the stream-ordered pool, as a plan's translated table */
		cudaError_t e = cudaMallocAsync(&b->d_arena, used, b->s);
		if (!e) e = cudaStreamSynchronize(b->s);
		if (e) {
			free(pieces.p);
			return sxs_cuda_fail(e, "sxsg_batch_create arena");
		}
	}
	/* per phase: translation launches per column class (stored rows, fused),
	 * then the per-pose launches (contraction of stored rows, sums over m) */
	bvec items = {NULL, 0, 0, sizeof(bitem)};
	size_t nn = np > 0 ? np : 1;
	sxsk_tr_job *tj = malloc(sizeof(sxsk_tr_job) * nn);
	sxsk_pc_job *pj = malloc(sizeof(sxsk_pc_job) * nn);
	sxsk_tf_job *fj = malloc(sizeof(sxsk_tf_job) * nn);
	sxsk_fr_job *rj = malloc(sizeof(sxsk_fr_job) * nn);
	int *jmap = malloc(sizeof(int) * nn), *fmap = malloc(sizeof(int) * nn);
	if (!tj || !pj || !fj || !rj || !jmap || !fmap) rc = sxs_fail(-5, "out of host memory");
	for (int ph = 0; ph < nphase && !rc; ph++) {
		int nj = 0, nf = 0;
		for (size_t k = 0; k < np; k++) {
			if (pc[k].phase != ph) continue;
			const bpiece *p = &pc[k];
			const sxs_plan_view *v = &b->v[p->plan];
			void *R = (char *)b->d_arena + p->off;
			int64_t p0 = v->h_cstart[p->c0], p1 = v->h_cstart[p->c1];
			int sb = v->tr_slices >= 1 ? v->tr_slices : SXSK_TP_SB;
			if (v->fused) {
				sxsk_tf_job *t = &fj[nf];
				memset(t, 0, sizeof(*t));
				t->U = v->U;
				t->tau = v->tauf;
				t->combo_zbg = v->combo + 3 * p->c0;
				t->slices = v->slices + 2 * p->s0;
				t->poses = v->poses;
				t->cstart = v->cstart;
				t->P = v->P;
				t->tw = v->tw;
				t->part = R;
				t->nslice = (int)(p->s1 - p->s0);
				t->cbase = (int)p->c0;
				t->L = v->L;
				t->nzt = v->nzt;
				t->sb = sb;
				t->pose_base = (int)p0;
				t->Q = v->Q;
				sxsk_fr_job *r = &rj[nf];
				memset(r, 0, sizeof(*r));
				r->poses = v->poses + p0;
				r->part = R;
				r->cst = v->cst;
				r->cross = v->cross;
				r->npose = (int)(p1 - p0);
				r->Q = v->Q;
				r->L = v->L;
				fmap[nf++] = (int)k;
				continue;
			}
			sxsk_tr_job *t = &tj[nj];
			memset(t, 0, sizeof(*t));
			t->U = v->U;
			t->tau = v->tauf;
			t->combo_zbg = v->combo + 3 * p->c0;
			t->slices = v->slices + 2 * p->s0;
			t->R = R;
			t->nslice = (int)(p->s1 - p->s0);
			t->cbase = (int)p->c0;
			t->ncombo = (int)(p->c1 - p->c0);
			t->L = v->L;
			t->nzt = v->nzt;
			t->sb = sb;
			t->Q = v->Q;
			sxsk_pc_job *q = &pj[nj];
			memset(q, 0, sizeof(*q));
			q->poses = v->poses + p0;
			q->P = v->P;
			q->R = R;
			q->tw = v->tw;
			q->cst = v->cst;
			q->cross = v->cross;
			q->npose = (int)(p1 - p0);
			q->combo_base = (int)p->c0;
			q->ncombo = (int)(p->c1 - p->c0);
			q->Q = v->Q;
			q->L = v->L;
			jmap[nj++] = (int)k;
		}
		int it_mode = b->flags & SXSG_BATCH_ITEMS;
		for (int NB = 4; NB <= 32 && !rc; NB += 4) {
			for (int j = 0; j < nj && !rc && it_mode; j++) {
				const bpiece *p = &pc[jmap[j]];
				const sxs_plan_view *v = &b->v[p->plan];
				rc = tr_items(&items, j, v, v->h_slices + 2 * p->s0, tj[j].nslice, tj[j].sb, NB);
			}
			if (!rc) rc = st_launch(st, 1, NB, ph, tj, sizeof(sxsk_tr_job) * nj, nj, &items, 0);
			for (int j = 0; j < nf && !rc && it_mode; j++) {
				const bpiece *p = &pc[fmap[j]];
				const sxs_plan_view *v = &b->v[p->plan];
				rc = tr_items(&items, j, v, v->h_slices + 2 * p->s0, fj[j].nslice, fj[j].sb, NB);
			}
			if (!rc) rc = st_launch(st, 4, NB, ph, fj, sizeof(sxsk_tf_job) * nf, nf, &items, 0);
		}
		for (int j = 0; j < nj && !rc && it_mode; j++) {
			const sxsk_pc_job *q = &pj[j];
			const sxs_plan_view *v = &b->v[pc[jmap[j]].plan];
			int bpt = (q->npose + 31) / 32;
			size_t i0 = items.n;
			for (int tt = 0; tt < v->NT && !rc; tt++)
				for (int pb = 0; pb < bpt && !rc; pb++) rc = add_item(&items, (double)v->NP, j, tt, pb, 0);
			job_cost(&items, i0);
		}
		if (!rc) rc = st_launch(st, 2, 0, ph, pj, sizeof(sxsk_pc_job) * nj, nj, &items, 0);
		for (int j = 0; j < nf && !rc && it_mode; j++) {
			long nblk = ((long)rj[j].npose * rj[j].Q + 127) / 128;
			size_t i0 = items.n;
			for (long k = 0; k < nblk && !rc; k++) rc = add_item(&items, (double)(rj[j].L + 1), j, (int)k, 0, 0);
			job_cost(&items, i0);
		}
		if (!rc) rc = st_launch(st, 5, 0, ph, rj, sizeof(sxsk_fr_job) * nf, nf, &items, 0);
	}
	free(items.p);
	free(tj);
	free(pj);
	free(fj);
	free(rj);
	free(jmap);
	free(fmap);
	free(pieces.p);
	return rc;
}

/* fit launch: items (dimer, group of poses) */
static int build_fit(sxsg_batch *b, bstage *st)
{
	bvec items = {NULL, 0, 0, sizeof(bitem)};
	sxsk_fit_job *jobs = calloc((size_t)b->n, sizeof(sxsk_fit_job));
	int rc = jobs ? 0 : sxs_fail(-5, "out of host memory"), nj = 0;
	b->fit_smem = 0;
	for (int i = 0; i < b->n && !rc; i++) {
		const sxs_plan_view *v = &b->v[i];
		if (v->npose <= 0) continue;
		sxsk_fit_job *J = &jobs[nj];
		size_t smem = 0;
		int e = sxsk_fit_df_shape(v->Q, v->n1, v->n2, &J->tp, &J->ppb, &J->qc, &J->gsm, &smem);
		if (e) {
			rc = sxs_fail(-2, "sxsg_batch_create: plan %d: no block shape fits its fit grid", i);
			break;
		}
		if (smem > b->fit_smem) b->fit_smem = smem;
		J->cross = (const float2 *)v->cross;
		J->order = NULL;
		J->fc = v->fc;
		J->gdf = v->gdf;
		J->c1g = v->c1g;
		J->c2g = v->c2g;
		J->chi = v->chi;
		J->c1 = v->c1;
		J->c2 = v->c2;
		J->cell = v->cell;
		J->grid = NULL;
		J->a0sum = v->a0sum;
		J->peak = v->peak;
		J->slot0 = 0;
		J->nslot = (int)v->npose;
		J->Q = v->Q;
		J->n1 = v->n1;
		J->n2 = v->n2;
		int ngroup = (J->nslot + J->ppb - 1) / J->ppb;
		double cost = (double)v->Q * ((v->n1 + J->tp - 1) / J->tp) * v->n2;
		size_t i0 = items.n;
		for (int g = 0; g < ngroup && !rc; g++) rc = add_item(&items, cost, nj, g, 0, 0);
		job_cost(&items, i0);
		nj++;
	}
	if (!rc) rc = st_launch(st, 3, 0, -1, jobs, sizeof(sxsk_fit_job) * nj, nj, &items, 1);
	free(jobs);
	free(items.p);
	return rc;
}

/* does column class NB hold an m for L (translate_col_launch's range) */
static int class_used(int L, int NB)
{
	int K = L + 1, m_hi = K - (NB - 3), m_lo = K - NB;
	if (m_hi > L) m_hi = L;
	if (m_lo < 0) m_lo = 0;
	return m_hi >= m_lo;
}

/* The translation and per-pose launches of a phase without work items: the
 * single-dimer kernels, one launch per piece (and column class), read from
 * the host copy of the jobs.  *nk += the kernels launched. */
static int launch_pieces(const blaunch *L, const char *hbase, int *nk, cudaStream_t s)
{
	const char *hj = hbase + L->jobs_off;
	int rc = 0;
	for (int j = 0; j < L->njobs && !rc; j++) {
		if (L->kind == 1) {
			const sxsk_tr_job *t = (const sxsk_tr_job *)hj + j;
			if (!class_used(t->L, L->arg)) continue;
			rc = sxsk_translate_class(t->U, t->tau, t->combo_zbg, t->slices, t->nslice, t->cbase, t->ncombo, t->nzt,
			                          t->Q, t->L, t->R, t->sb, L->arg, s);
		} else if (L->kind == 4) {
			const sxsk_tf_job *t = (const sxsk_tf_job *)hj + j;
			if (!class_used(t->L, L->arg)) continue;
			rc = sxsk_translate_fused_class(t->U, t->tau, t->combo_zbg, t->slices, t->nslice, t->cbase, t->nzt, t->Q,
			                                t->L, t->sb, t->poses, t->cstart, t->pose_base, t->P, t->tw, t->part,
			                                L->arg, s);
		} else if (L->kind == 2) {
			const sxsk_pc_job *q = (const sxsk_pc_job *)hj + j;
			rc = sxsk_pose_cross(q->poses, q->npose, q->combo_base, q->ncombo, q->P, q->R, q->tw, q->cst, q->Q, q->L,
			                     q->cross, 1, s);
		} else {
			const sxsk_fr_job *r = (const sxsk_fr_job *)hj + j;
			rc = sxsk_fused_reduce(r->poses, r->npose, r->part, r->Q, r->L, r->cst, r->cross, s);
		}
		(*nk)++;
	}
	return rc;
}

static int launch_one(sxsg_batch *b, const blaunch *L, int *ctr, const char *hbase, int *nk, cudaStream_t s)
{
	char *base = b->d_buf;
	const void *jobs = base + L->jobs_off, *items = base + L->items_off;
	int *c = ctr ? ctr + L->ctr : NULL;   /* NULL: one block per item */
	int k = L->kind;
	if (!(b->flags & SXSG_BATCH_ITEMS) && (k == 1 || k == 2 || k == 4 || k == 5)) return launch_pieces(L, hbase, nk, s);
	if (L->nitems > 0) (*nk)++;
	switch (k) {
	case 0: return sxsk_rotate_batch(jobs, items, L->nitems, L->arg & 0xff, L->arg >> 8, c, s);
	case 1: return sxsk_translate_batch(jobs, items, L->nitems, L->arg, c, s);
	case 2: return sxsk_pose_cross_batch(jobs, items, L->nitems, c, s);
	case 4: return sxsk_translate_fused_batch(jobs, items, L->nitems, L->arg, c, s);
	case 5: return sxsk_fused_reduce_batch(jobs, items, L->nitems, c, s);
	default: return sxsk_fit_grid_df_batch(jobs, items, L->nitems, b->fit_smem, c, s);
	}
}

/* The graph, captured from b->s: counters zeroed; the per-z tables on two
 * branches beside the rotation launches; then the phases on two lanes:
 * the translation launches of a phase on one stream per column class (the
 * classes of a phase run side by side, each class's phases in order), the
 * per-pose launch of a phase on the pose lane once its translations are
 * done.  A phase's translations wait for the per-pose launch of the last
 * phase that used the same arena half: with SXSG_BATCH_OVERLAP (two
 * halves) the translations of phase k + 1 run beside the per-pose work of
 * phase k.  The fit follows the last per-pose launch. */
static int capture(sxsg_batch *b, const blaunch *ls, int nl, int *ctr, const char *hbase)
{
	cudaStream_t s = b->s, ps = b->ps;
	int rc = 0, nk = 0;
	int *c = (b->flags & SXSG_BATCH_PERSISTENT) ? ctr : NULL;
	SXS_CU(cudaStreamBeginCapture(s, cudaStreamCaptureModeRelaxed));
	cudaError_t e = cudaMemsetAsync(ctr, 0, sizeof(int) * (size_t)(nl > 0 ? nl : 1), s);
	if (!e) e = cudaEventRecordWithFlags(b->ev[0], s, cudaEventRecordExternal);
	/* per-z tables of every dimer on two branches */
	if (!e) e = cudaEventRecord(b->fork, s);
	for (int k = 0; k < 2 && !e; k++) e = cudaStreamWaitEvent(b->br[k], b->fork, 0);
	for (int i = 0; i < b->n && !e && !rc; i++) {
		if (b->v[i].nzt <= 0) continue;
		rc = sxs_plan_ztables_on(b->plans[i], b->br[i & 1]);
		nk += 3;
	}
	int li = 0;
	while (li < nl && ls[li].kind == 0 && !e && !rc) {
		rc = launch_one(b, &ls[li], c, hbase, &nk, s);
		li++;
	}
	for (int k = 0; k < 2 && !e; k++) {
		e = cudaEventRecord(b->join[k], b->br[k]);
		if (!e) e = cudaStreamWaitEvent(s, b->join[k], 0);
	}
	if (!e) e = cudaEventRecordWithFlags(b->ev[1], s, cudaEventRecordExternal);
	/* phases */
	if (!e) e = cudaEventRecord(b->fork, s);
	for (int k = 0; k < SXSB_BR && !e; k++) e = cudaStreamWaitEvent(b->br[k], b->fork, 0);
	if (!e) e = cudaStreamWaitEvent(ps, b->fork, 0);
	int halves = (b->flags & SXSG_BATCH_OVERLAP) ? 2 : 1;
	for (int ph = 0; ph < b->nphase && !e && !rc; ph++) {
		int h = ph % halves;
		while (li < nl && (ls[li].kind == 1 || ls[li].kind == 4) && ls[li].phase == ph && !e && !rc) {
			int cls = ls[li].arg / 4 - 1;
			cudaStream_t bs = b->br[cls];
			if (ph >= halves) e = cudaStreamWaitEvent(bs, b->evpose[h], 0);
			if (!e) rc = launch_one(b, &ls[li], c, hbase, &nk, bs);
			if (!e && !rc) e = cudaEventRecord(b->join[cls], bs);
			if (!e) e = cudaStreamWaitEvent(ps, b->join[cls], 0);
			li++;
		}
		while (li < nl && (ls[li].kind == 2 || ls[li].kind == 5) && ls[li].phase == ph && !e && !rc) {
			rc = launch_one(b, &ls[li], c, hbase, &nk, ps);
			li++;
		}
		if (!e && !rc) e = cudaEventRecord(b->evpose[h], ps);
	}
	/* every lane back into the origin stream */
	for (int k = 0; k < SXSB_BR && !e; k++) {
		e = cudaEventRecord(b->join[k], b->br[k]);
		if (!e) e = cudaStreamWaitEvent(s, b->join[k], 0);
	}
	if (!e) e = cudaEventRecord(b->evpose[0], ps);
	if (!e) e = cudaStreamWaitEvent(s, b->evpose[0], 0);
	if (!e) e = cudaEventRecordWithFlags(b->ev[2], s, cudaEventRecordExternal);
	if (li < nl && ls[li].kind == 3 && !e && !rc) {
		rc = launch_one(b, &ls[li], c, hbase, &nk, s);
		li++;
	}
	if (!e) e = cudaEventRecordWithFlags(b->ev[3], s, cudaEventRecordExternal);
	cudaGraph_t g = NULL;
	cudaError_t e2 = cudaStreamEndCapture(s, &g);
	if (!e) e = e2;
	if (rc || e) {
		if (g) cudaGraphDestroy(g);
		return rc ? rc : sxs_cuda_fail(e, "sxsg_batch_create capture");
	}
	if (li != nl) {
		cudaGraphDestroy(g);
		return sxs_fail(-2, "sxsg_batch_create: launch list out of order");
	}
	b->graph = g;
	e = cudaGraphInstantiate(&b->exec, g, 0);
	if (e) return sxs_cuda_fail(e, "sxsg_batch_create instantiate");
	b->nkern = nk;
	return 0;
}

int sxsg_batch_create(sxsg_plan *const *plans, int nplan, int fit_mode, size_t arena_bytes, int flags,
                      sxsg_batch **out)
{
	if (!plans || nplan <= 0 || !out) return sxs_fail(-2, "sxsg_batch_create: bad arguments");
	if (flags & ~(SXSG_BATCH_PERSISTENT | SXSG_BATCH_OVERLAP | SXSG_BATCH_ITEMS))
		return sxs_fail(-2, "sxsg_batch_create: unknown flags 0x%x", flags);
	if (fit_mode != SXSG_FIT_GRID && fit_mode != SXSG_FIT_NONE)
		return sxs_fail(-2, "sxsg_batch_create: fit mode must be SXSG_FIT_GRID or SXSG_FIT_NONE");
	*out = NULL;
	int rc = sxs_ensure_init();
	if (rc) return rc;
	sxsg_batch *b = calloc(1, sizeof(*b));
	if (!b) return sxs_fail(-5, "out of host memory");
	b->n = nplan;
	b->fit_mode = fit_mode;
	b->flags = flags;
	b->plans = malloc(sizeof(sxsg_plan *) * (size_t)nplan);
	b->v = calloc((size_t)nplan, sizeof(sxs_plan_view));
	if (!b->plans || !b->v) {
		sxsg_batch_destroy(b);
		return sxs_fail(-5, "out of host memory");
	}
	for (int i = 0; i < nplan && !rc; i++) {
		b->plans[i] = plans[i];
		if (!plans[i]) {
			rc = sxs_fail(-2, "sxsg_batch_create: plan %d is NULL", i);
			break;
		}
		for (int k = 0; k < i; k++)
			if (plans[k] == plans[i]) rc = sxs_fail(-2, "sxsg_batch_create: plan %d listed twice", i);
		if (!rc) rc = sxs_plan_batch_view(plans[i], &b->v[i]);
		const sxs_plan_view *v = &b->v[i];
		if (!rc && !v->fp32) rc = sxs_fail(-2, "sxsg_batch_create: plan %d is not mixed precision", i);
		if (!rc && v->L + 1 > 32) rc = sxs_fail(-2, "sxsg_batch_create: plan %d has L = %d > 31", i, v->L);
		if (!rc && v->ext_tables) rc = sxs_fail(-2, "sxsg_batch_create: plan %d uses caller rotation tables", i);
		if (!rc && fit_mode == SXSG_FIT_GRID && (v->n1 <= 0 || v->n2 <= 0))
			rc = sxs_fail(-2, "sxsg_batch_create: plan %d has no (c1, c2) grid", i);
		if (!rc && sxsk_rotate_group(v->L, v->rot_gamma) == 0)
			rc = sxs_fail(-2, "sxsg_batch_create: plan %d: no rotation group for its tile choice", i);
		b->nposes += v->npose;
	}
	cudaError_t e = cudaSuccess;
	if (!rc) e = cudaStreamCreateWithFlags(&b->s, cudaStreamNonBlocking);
	if (!e && !rc) e = cudaStreamCreateWithFlags(&b->ps, cudaStreamNonBlocking);
	for (int k = 0; k < 2 && !e && !rc; k++) e = cudaEventCreateWithFlags(&b->evpose[k], cudaEventDisableTiming);
	int plo = 0, phi = 0;
	if (!e && !rc) e = cudaDeviceGetStreamPriorityRange(&plo, &phi);
	for (int k = 0; k < SXSB_BR && !e && !rc; k++) {
		/* the per-z tables (branches 0 and 1: FP64 pipe) at the highest
		 * priority: their blocks take SM slots as they free up beside the
		 * rotation blocks (FP32 pipe) instead of waiting for the rotation
		 * grids to be dispatched */
		e = cudaStreamCreateWithPriority(&b->br[k], cudaStreamNonBlocking, k < 2 ? phi : plo);
		if (!e) e = cudaEventCreateWithFlags(&b->join[k], cudaEventDisableTiming);
	}
	if (!e && !rc) e = cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming);
	for (int k = 0; k < 4 && !e && !rc; k++) e = cudaEventCreate(&b->ev[k]);
	if (e && !rc) rc = sxs_cuda_fail(e, "sxsg_batch_create streams");
	bstage st = {NULL, 0, 0, {NULL, 0, 0, sizeof(blaunch)}};
	if (!rc) rc = build_rotations(b, &st);
	if (!rc) rc = build_phases(b, &st, arena_bytes);
	if (!rc && fit_mode == SXSG_FIT_GRID) rc = build_fit(b, &st);
	int nl = (int)st.launches.n;
	size_t ctr_off = al(st.used);
	if (!rc) {
		e = cudaMalloc(&b->d_buf, ctr_off + sizeof(int) * (size_t)(nl > 0 ? nl : 1));
		if (!e && st.used) e = cudaMemcpy(b->d_buf, st.h, st.used, cudaMemcpyHostToDevice);
		if (e) rc = sxs_cuda_fail(e, "sxsg_batch_create work lists");
	}
	if (!rc) {
		const blaunch *ls = st.launches.p;
		for (int k = 0; k < nl; k++) b->nitems += ls[k].nitems;
		b->nlaunch = nl;
		rc = capture(b, ls, nl, (int *)((char *)b->d_buf + ctr_off), st.h);
	}
	free(st.h);
	free(st.launches.p);
	if (rc) {
		sxsg_batch_destroy(b);
		return rc;
	}
	*out = b;
	return 0;
}

int sxsg_batch_run(sxsg_batch *b)
{
	if (!b || !b->exec) return sxs_fail(-2, "sxsg_batch_run: no batch");
	cudaEvent_t a, z;
	SXS_CU(cudaEventCreate(&a));
	cudaError_t e = cudaEventCreate(&z);
	if (e) {
		cudaEventDestroy(a);
		return sxs_cuda_fail(e, "sxsg_batch_run events");
	}
	e = cudaEventRecord(a, b->s);
	if (!e) e = cudaGraphLaunch(b->exec, b->s);
	if (!e) e = cudaEventRecord(z, b->s);
	if (!e) e = cudaEventSynchronize(z);
	if (!e) e = cudaGetLastError();
	float t[4] = {0, 0, 0, 0};
	if (!e) {
		cudaEventElapsedTime(&t[0], b->ev[0], b->ev[1]);
		cudaEventElapsedTime(&t[1], b->ev[1], b->ev[2]);
		cudaEventElapsedTime(&t[2], b->ev[2], b->ev[3]);
		cudaEventElapsedTime(&t[3], a, z);
	}
	cudaEventDestroy(a);
	cudaEventDestroy(z);
	if (e) return sxs_cuda_fail(e, "sxsg_batch_run");
	for (int k = 0; k < 4; k++) b->ms[k] = t[k];
	float pms[5] = {t[0], t[1], 0.0f, t[2], t[3]};
	for (int i = 0; i < b->n; i++) sxs_plan_mark_run(b->plans[i], b->fit_mode, pms);
	sxs_count_launches(b->nkern);
	return 0;
}

int sxsg_batch_stats_get(const sxsg_batch *b, sxsg_batch_stats *st)
{
	if (!b || !st) return sxs_fail(-2, "sxsg_batch_stats_get: bad arguments");
	memset(st, 0, sizeof(*st));
	st->plans = b->n;
	st->phases = b->nphase;
	st->launches = b->nkern;
	st->items = b->nitems;
	st->poses = b->nposes;
	st->arena_bytes = b->arena;
	for (int k = 0; k < 4; k++) st->ms[k] = b->ms[k];
	return 0;
}
