/*
 * Serving loop: a persistent pool of host workers that keeps one GB300 busy
 * with many scoring jobs at once.
 *
 *  - Jobs are admitted in arrival order (FIFO) as device memory frees up:
 *    a job's footprint (plan tables, per-z tables, pose lists, outputs, its
 *    translated-table chunk) plus any rotation tables it has to add to the
 *    cache must fit under the server's HBM cap.  A job larger than the cap
 *    runs alone.
 *  - Each worker owns a CUDA stream; admitted jobs run concurrently on the
 *    device (continuous batching: a job that arrives while others run is
 *    started as soon as a worker and memory are free, and its kernels
 *    interleave with theirs).  Plans allocate stream-ordered, so one job's
 *    frees never stall another's kernels.
 *  - Rotation tables (receptor P, ligand U) of molecules with a nonzero
 *    caller key are cached on the device, keyed by a hash of the
 *    coefficients themselves, the caller's key, L, the q grid, the twiddle
 *    variant and the precision; a job whose receptor (or ligand) table is
 *    cached and complete skips that rotation.  A table is shared only once
 *    the job that filled it has finished on the device (its stream was
 *    synchronised before the entry is marked valid); a job that finds its
 *    table still being filled by another running job fills a private copy.
 *    Unreferenced entries are evicted least recently used when admission
 *    needs the memory.
 *  - Results are bitwise those of the same job run alone: every kernel is
 *    deterministic, and the only device state jobs share is complete
 *    rotation tables that they read and never write.
 */
#define _XOPEN_SOURCE 700
#include <pthread.h>
#include <stdlib.h>
#include <string.h>
#include <time.h>

#include "sxs_internal.h"

typedef struct sxs_job {
	int64_t ticket;
	double *A, *B, *q, *z, *a, *c1g, *c2g;
	int64_t *index;
	int Q, nz, L, n1, n2, skip, fit_mode, precision, nzt;
	int64_t n;
	double mult, peak;
	uint64_t keyA, keyB;
	uint64_t kP, kU;            /* rotation-table cache keys (0: not cached) */
	size_t bytes, rbudget, tbytes;
	double t_submit, t_start, t_end;
	double *chi, *c1, *c2;
	int status;                 /* 0 queued, 1 running, 2 done */
	int rc;
	char err[256];
	struct sxs_job *next;
} sxs_job;

typedef struct sxs_tentry {
	uint64_t key;
	void *d;
	size_t bytes;
	int valid;                  /* filled by a job that has finished on the device */
	int refs, priv;
	uint64_t stamp;
	struct sxs_tentry *next;
} sxs_tentry;

struct sxsg_server {
	pthread_mutex_t mu;
	pthread_cond_t cv_work, cv_done;
	sxs_job *head, *tail;
	sxs_job **jobs;
	int64_t njobs, capjobs;
	size_t cap, used;
	int nworkers, stop;
	pthread_t *th;
	cudaStream_t *streams;
	sxs_tentry *cache;
	size_t cache_bytes;
	uint64_t clock, priv_key;
	int64_t hits, misses, completed, poses;
};

typedef struct {
	sxsg_server *s;
	int id;
} sxs_winfo;

static double now_ms(void)
{
	struct timespec ts;
	clock_gettime(CLOCK_MONOTONIC, &ts);
	return ts.tv_sec * 1e3 + ts.tv_nsec * 1e-6;
}

static uint64_t fnv(uint64_t h, const void *p, size_t n)
{
	const unsigned char *b = p;
	for (size_t i = 0; i < n; i++) {
		h ^= b[i];
		h *= 1099511628211ull;
	}
	return h;
}

/* 64-bit digest of n doubles, word by word (multiply-xorshift mixing) */
static uint64_t digest(const double *x, size_t n)
{
	uint64_t h = 0x243f6a8885a308d3ull ^ (uint64_t)n;
	for (size_t i = 0; i < n; i++) {
		uint64_t w;
		memcpy(&w, x + i, sizeof(w));
		h ^= w;
		h *= 0x9e3779b97f4a7c15ull;
		h ^= h >> 29;
	}
	return h;
}

/* Cache key of a rotation table: the coefficients' digest (so a reused
 * caller key with other coefficients never aliases), the caller's key, the
 * role (P or U) and everything else the table depends on.  0 = not cached. */
static uint64_t table_key(uint64_t mol, int role, const sxs_job *j, const double *coef)
{
	if (!mol) return 0;
	int K = j->L + 1;
	uint64_t h = 1469598103934665603ull;
	int v[5] = {role, j->L, j->Q, j->skip == 1, j->precision};
	uint64_t d = digest(coef, (size_t)3 * j->Q * K * K * 2);
	h = fnv(h, &mol, sizeof(mol));
	h = fnv(h, &d, sizeof(d));
	h = fnv(h, v, sizeof(v));
	h = fnv(h, j->q, sizeof(double) * j->Q);
	return h ? h : 1;
}

/* a shared entry of this key, complete or still being filled */
static sxs_tentry *cache_find(sxsg_server *s, uint64_t key)
{
	for (sxs_tentry *e = s->cache; e; e = e->next)
		if (e->key == key && !e->priv) return e;
	return NULL;
}

/* a shared entry of this key that a job may read */
static sxs_tentry *cache_find_valid(sxsg_server *s, uint64_t key)
{
	sxs_tentry *e = key ? cache_find(s, key) : NULL;
	return e && e->valid ? e : NULL;
}

/* free unreferenced entries, least recently used first, until `need` more
 * bytes fit beside the running jobs; returns whether they fit */
static int cache_make_room(sxsg_server *s, size_t need, cudaStream_t st)
{
	while (s->used + s->cache_bytes + need > s->cap) {
		sxs_tentry *victim = NULL, **vp = NULL;
		for (sxs_tentry **pp = &s->cache; *pp; pp = &(*pp)->next)
			if ((*pp)->refs == 0 && (!victim || (*pp)->stamp < victim->stamp)) {
				victim = *pp;
				vp = pp;
			}
		if (!victim) return 0;
		*vp = victim->next;
		s->cache_bytes -= victim->bytes;
		cudaFreeAsync(victim->d, st);
		free(victim);
	}
	return 1;
}

/* bytes a job adds beyond its own footprint: the tables it must fill */
static size_t job_table_need(sxsg_server *s, const sxs_job *j)
{
	size_t need = 0;
	if (!cache_find_valid(s, j->kP)) need += j->tbytes;
	if (!cache_find_valid(s, j->kU)) need += j->tbytes;
	return need;
}

/* A table for a job: a complete shared entry (read only), else a new one
 * that this job fills.  The new entry is shared (others find it once it is
 * valid) unless the key is 0 or a shared entry of the key is already being
 * filled by another running job, whose rotation may still be in flight on
 * its own stream: then the new entry is private to this job. */
static sxs_tentry *cache_acquire(sxsg_server *s, uint64_t key, size_t bytes, cudaStream_t st, int *err)
{
	sxs_tentry *e = cache_find_valid(s, key);
	if (e) {
		e->refs++;
		e->stamp = ++s->clock;
		s->hits++;
		return e;
	}
	int priv = key == 0 || cache_find(s, key) != NULL;
	s->misses++;
	e = calloc(1, sizeof(*e));
	e->key = priv ? ++s->priv_key : key;
	e->priv = priv;
	e->bytes = bytes;
	e->refs = 1;
	e->stamp = ++s->clock;
	cudaError_t ce = cudaMallocAsync(&e->d, bytes, st);
	if (!ce) ce = cudaMemsetAsync(e->d, 0, bytes, st);
	if (ce) {
		free(e);
		*err = (int)ce;
		return NULL;
	}
	e->next = s->cache;
	s->cache = e;
	s->cache_bytes += bytes;
	return e;
}

/* Called after the job's stream was synchronised: a table it filled is
 * complete on the device, so marking it valid lets jobs on other streams
 * read it without further ordering. */
static void cache_release(sxsg_server *s, sxs_tentry *e, int valid, cudaStream_t st)
{
	if (!e) return;
	e->refs--;
	if (valid) e->valid = 1;
	if (e->priv || (!e->valid && e->refs == 0)) {
		for (sxs_tentry **pp = &s->cache; *pp; pp = &(*pp)->next)
			if (*pp == e) {
				*pp = e->next;
				break;
			}
		s->cache_bytes -= e->bytes;
		cudaFreeAsync(e->d, st);
		free(e);
	}
}

static int job_fail(sxs_job *j, int rc)
{
	j->rc = rc;
	snprintf(j->err, sizeof(j->err), "%s", sxsg_last_error());
	return rc;
}

static int run_job(sxs_job *j, cudaStream_t st, sxs_tentry *tp, sxs_tentry *tu, int *P_ok, int *U_ok)
{
	sxsg_plan *p = NULL;
	int rc = sxs_plan_create_on(&p, j->A, j->B, j->q, j->Q, j->z, j->nz, j->L, j->a, j->mult, j->peak, j->c1g,
	                            j->n1, j->c2g, j->n2, j->precision, st, 1);
	if (rc) return job_fail(j, rc);
	sxs_plan_set_tables(p, tp->d, tp->valid, tu->d, tu->valid);
	sxsg_plan_set_budget(p, j->rbudget);
	rc = sxsg_plan_set_poses(p, j->index, j->n, j->skip);
	if (!rc) rc = sxsg_plan_run(p, j->fit_mode);
	if (!rc) rc = sxsg_plan_results(p, j->chi, j->c1, j->c2, NULL, NULL, NULL);
	*P_ok = *U_ok = rc == 0;
	if (rc) job_fail(j, rc);
	sxsg_plan_destroy(p);
	return rc;
}

static void *worker(void *arg)
{
	sxs_winfo *w = arg;
	sxsg_server *s = w->s;
	cudaStream_t st = s->streams[w->id];
	free(w);
	sxs_ensure_init();
	pthread_mutex_lock(&s->mu);
	for (;;) {
		sxs_job *j = NULL;
		while (!j) {
			if (s->head) {
				sxs_job *h = s->head;
				size_t need = h->bytes + job_table_need(s, h);
				int running = s->used > 0;
				if (cache_make_room(s, need, st) || !running) j = h;
			}
			if (j) break;
			if (s->stop && !s->head) break;
			pthread_cond_wait(&s->cv_work, &s->mu);
		}
		if (!j) break;
		s->head = j->next;
		if (!s->head) s->tail = NULL;
		s->used += j->bytes;
		j->status = 1;
		j->t_start = now_ms();
		int err = 0;
		sxs_tentry *tp = cache_acquire(s, j->kP, j->tbytes, st, &err);
		sxs_tentry *tu = tp ? cache_acquire(s, j->kU, j->tbytes, st, &err) : NULL;
		pthread_mutex_unlock(&s->mu);
		int P_ok = 0, U_ok = 0;
		if (tp && tu) {
			run_job(j, st, tp, tu, &P_ok, &U_ok);
		} else {
			j->rc = -100 - err;
			snprintf(j->err, sizeof(j->err), "serving: rotation table allocation failed (%s)",
			         cudaGetErrorString((cudaError_t)err));
		}
		cudaStreamSynchronize(st);
		pthread_mutex_lock(&s->mu);
		cache_release(s, tp, P_ok, st);
		cache_release(s, tu, U_ok, st);
		s->used -= j->bytes;
		j->t_end = now_ms();
		j->status = 2;
		s->completed++;
		if (j->rc == 0) s->poses += j->n;
		free(j->A); free(j->B); free(j->q); free(j->z); free(j->a); free(j->c1g); free(j->c2g); free(j->index);
		j->A = j->B = j->q = j->z = j->a = j->c1g = j->c2g = NULL;
		j->index = NULL;
		pthread_cond_broadcast(&s->cv_done);
		pthread_cond_broadcast(&s->cv_work);
	}
	pthread_mutex_unlock(&s->mu);
	return NULL;
}

int sxsg_server_create(sxsg_server **out, size_t hbm_cap, int max_active)
{
	if (!out || max_active < 1 || max_active > 64) return sxs_fail(-2, "sxsg_server_create: bad arguments");
	int rc = sxs_ensure_init();
	if (rc) return rc;
	sxsg_server *s = calloc(1, sizeof(*s));
	if (!s) return sxs_fail(-5, "out of host memory");
	pthread_mutex_init(&s->mu, NULL);
	pthread_cond_init(&s->cv_work, NULL);
	pthread_cond_init(&s->cv_done, NULL);
	if (hbm_cap == 0) {
		size_t fr = 0, tot = 0;
		cudaMemGetInfo(&fr, &tot);
		hbm_cap = fr / 10 * 9;
	}
	s->cap = hbm_cap;
	s->nworkers = max_active;
	s->th = calloc(max_active, sizeof(pthread_t));
	s->streams = calloc(max_active, sizeof(cudaStream_t));
	if (!s->th || !s->streams) {
		free(s->th); free(s->streams); free(s);
		return sxs_fail(-5, "out of host memory");
	}
	for (int i = 0; i < max_active; i++) {
		cudaError_t e = cudaStreamCreateWithFlags(&s->streams[i], cudaStreamNonBlocking);
		if (e) {
			for (int k = 0; k < i; k++) cudaStreamDestroy(s->streams[k]);
			free(s->th); free(s->streams); free(s);
			return sxs_cuda_fail(e, "sxsg_server_create stream");
		}
	}
	for (int i = 0; i < max_active; i++) {
		sxs_winfo *w = malloc(sizeof(*w));
		if (w) {
			w->s = s;
			w->id = i;
		}
		if (!w || pthread_create(&s->th[i], NULL, worker, w)) {
			/* stop and join the workers already started, then release */
			free(w);
			int started = i;
			for (int k = started; k < max_active; k++) cudaStreamDestroy(s->streams[k]);
			s->nworkers = started;
			sxsg_server_destroy(s);
			return sxs_fail(-5, "sxsg_server_create: cannot start worker %d", i);
		}
	}
	*out = s;
	return 0;
}

static void *dup_arr(const void *p, size_t n)
{
	if (!p || n == 0) return NULL;
	void *d = malloc(n);
	memcpy(d, p, n);
	return d;
}

static void job_free(sxs_job *j)
{
	if (!j) return;
	free(j->A); free(j->B); free(j->q); free(j->z); free(j->a); free(j->c1g); free(j->c2g); free(j->index);
	free(j->chi); free(j->c1); free(j->c2); free(j);
}

int64_t sxsg_server_submit(sxsg_server *s, const sxsg_request *r)
{
	if (!s || !r || !r->A || !r->B || !r->qvals || r->qnum <= 0 || r->qnum > 1024 || !r->zvals || r->znum <= 0 ||
	    !r->a || r->L < 1 || r->L > SXS_LMAX || r->n < 0 || (r->n > 0 && !r->index) || r->n > INT32_MAX)
		return sxs_fail(-2, "sxsg_server_submit: bad request");
	if (r->fit_mode == SXSG_FIT_GRID && (r->n1 <= 0 || r->n2 <= 0 || !r->c1grid || !r->c2grid))
		return sxs_fail(-2, "sxsg_server_submit: grid fit needs a (c1, c2) grid");
	if (r->precision != SXSG_FP64 && r->precision != SXSG_MIXED)
		return sxs_fail(-2, "sxsg_server_submit: unknown precision");
	int L = r->L, Q = r->qnum, K = L + 1, N = 2 * L + 1;
	size_t spf = sizeof(double) * 3 * Q * K * K * 2;
	sxs_job *j = calloc(1, sizeof(*j));
	if (!j) return sxs_fail(-5, "out of host memory");
	j->A = dup_arr(r->A, spf);
	j->B = dup_arr(r->B, spf);
	j->q = dup_arr(r->qvals, sizeof(double) * Q);
	j->z = dup_arr(r->zvals, sizeof(double) * r->znum);
	j->a = dup_arr(r->a, sizeof(double) * 6 * Q);
	j->c1g = dup_arr(r->c1grid, sizeof(double) * (r->n1 > 0 ? r->n1 : 0));
	j->c2g = dup_arr(r->c2grid, sizeof(double) * (r->n2 > 0 ? r->n2 : 0));
	j->index = dup_arr(r->index, sizeof(int64_t) * r->n);
	j->Q = Q; j->nz = r->znum; j->L = L; j->n1 = r->n1; j->n2 = r->n2; j->skip = r->skip;
	j->fit_mode = r->fit_mode; j->precision = r->precision; j->n = r->n; j->mult = r->mult; j->peak = r->peak;
	j->keyA = r->keyA;
	j->keyB = r->keyB;
	j->kP = table_key(r->keyA, 0, j, j->A);
	j->kU = table_key(r->keyB, 1, j, j->B);
	size_t n = r->n > 0 ? (size_t)r->n : 1;
	j->chi = malloc(sizeof(double) * n);
	j->c1 = malloc(sizeof(double) * n);
	j->c2 = malloc(sizeof(double) * n);
	/* touched z and the combo bound for the footprint */
	char *zu = calloc(r->znum, 1);
	if (!j->A || !j->B || !j->q || !j->z || !j->a || (r->c1grid && r->n1 > 0 && !j->c1g) ||
	    (r->c2grid && r->n2 > 0 && !j->c2g) || (r->n > 0 && !j->index) || !j->chi || !j->c1 || !j->c2 || !zu) {
		free(zu);
		job_free(j);
		return sxs_fail(-5, "out of host memory");
	}
	int64_t per_z = (int64_t)K * K * N * N * N;
	int nzt = 0;
	for (int64_t i = 0; i < r->n; i++) {
		int64_t zi = r->index[i] / per_z;
		if (zi >= 0 && zi < r->znum && !zu[zi]) {
			zu[zi] = 1;
			nzt++;
		}
	}
	free(zu);
	j->nzt = nzt;
	int64_t combos = (int64_t)nzt * K * N;
	if (combos > r->n) combos = r->n;
	size_t rfull = (size_t)combos * sxs_plan_combo_bytes(L, Q, r->precision);
	size_t rcap = s->cap / (4 * (size_t)s->nworkers);
	if (rcap < ((size_t)64 << 20)) rcap = (size_t)64 << 20;
	j->rbudget = rfull < rcap ? rfull : rcap;
	if (j->rbudget < sxs_plan_combo_bytes(L, Q, r->precision) * 16)
		j->rbudget = sxs_plan_combo_bytes(L, Q, r->precision) * 16;
	j->tbytes = sxs_plan_table_bytes(L, Q, r->precision);
	j->bytes = sxs_plan_base_bytes(L, Q, nzt, r->n, r->n1, r->precision, r->fit_mode) + j->rbudget;
	j->t_submit = now_ms();
	pthread_mutex_lock(&s->mu);
	if (s->stop) {
		pthread_mutex_unlock(&s->mu);
		job_free(j);
		return sxs_fail(-2, "sxsg_server_submit: server is shutting down");
	}
	if (s->njobs == s->capjobs) {
		int64_t cap = s->capjobs ? 2 * s->capjobs : 64;
		sxs_job **nj = realloc(s->jobs, sizeof(sxs_job *) * cap);
		if (!nj) {
			pthread_mutex_unlock(&s->mu);
			job_free(j);
			return sxs_fail(-5, "out of host memory");
		}
		s->jobs = nj;
		s->capjobs = cap;
	}
	j->ticket = s->njobs;
	s->jobs[s->njobs++] = j;
	if (s->tail) s->tail->next = j;
	else s->head = j;
	s->tail = j;
	pthread_cond_broadcast(&s->cv_work);
	pthread_mutex_unlock(&s->mu);
	return j->ticket;
}

int sxsg_server_poll(sxsg_server *s, int64_t ticket)
{
	if (!s || ticket < 0) return sxs_fail(-2, "sxsg_server_poll: bad ticket");
	pthread_mutex_lock(&s->mu);
	int st = ticket < s->njobs && s->jobs[ticket] ? (s->jobs[ticket]->status == 2) : -1;
	pthread_mutex_unlock(&s->mu);
	return st < 0 ? sxs_fail(-2, "sxsg_server_poll: unknown or collected ticket") : st;
}

int sxsg_server_wait(sxsg_server *s, int64_t ticket, double *chi, double *c1, double *c2, double *ms3)
{
	if (!s || ticket < 0) return sxs_fail(-2, "sxsg_server_wait: bad ticket");
	pthread_mutex_lock(&s->mu);
	if (ticket >= s->njobs || !s->jobs[ticket]) {
		pthread_mutex_unlock(&s->mu);
		return sxs_fail(-2, "sxsg_server_wait: unknown or collected ticket");
	}
	sxs_job *j = s->jobs[ticket];
	while (j->status != 2) pthread_cond_wait(&s->cv_done, &s->mu);
	s->jobs[ticket] = NULL;
	pthread_mutex_unlock(&s->mu);
	int rc = j->rc;
	if (!rc) {
		if (chi) memcpy(chi, j->chi, sizeof(double) * j->n);
		if (c1) memcpy(c1, j->c1, sizeof(double) * j->n);
		if (c2) memcpy(c2, j->c2, sizeof(double) * j->n);
	} else {
		sxs_fail(rc, "%s", j->err);
	}
	if (ms3) {
		ms3[0] = j->t_start - j->t_submit;
		ms3[1] = j->t_end - j->t_start;
		ms3[2] = j->t_end - j->t_submit;
	}
	free(j->chi); free(j->c1); free(j->c2); free(j);
	return rc;
}

int sxsg_server_stats(sxsg_server *s, double *out8)
{
	if (!s || !out8) return sxs_fail(-2, "sxsg_server_stats: bad arguments");
	pthread_mutex_lock(&s->mu);
	int64_t queued = 0;
	for (sxs_job *j = s->head; j; j = j->next) queued++;
	int64_t entries = 0;
	for (sxs_tentry *e = s->cache; e; e = e->next) entries++;
	out8[0] = (double)s->completed;
	out8[1] = (double)s->poses;
	out8[2] = (double)queued;
	out8[3] = (double)s->used;
	out8[4] = (double)s->cache_bytes;
	out8[5] = (double)entries;
	out8[6] = (double)s->hits;
	out8[7] = (double)s->misses;
	pthread_mutex_unlock(&s->mu);
	return 0;
}

void sxsg_server_destroy(sxsg_server *s)
{
	if (!s) return;
	pthread_mutex_lock(&s->mu);
	s->stop = 1;
	pthread_cond_broadcast(&s->cv_work);
	pthread_mutex_unlock(&s->mu);
	for (int i = 0; i < s->nworkers; i++) pthread_join(s->th[i], NULL);
	for (int i = 0; i < s->nworkers; i++) cudaStreamSynchronize(s->streams[i]);
	while (s->cache) {
		sxs_tentry *e = s->cache;
		s->cache = e->next;
		cudaFree(e->d);
		free(e);
	}
	for (int64_t t = 0; t < s->njobs; t++)
		if (s->jobs[t]) {
			free(s->jobs[t]->chi); free(s->jobs[t]->c1); free(s->jobs[t]->c2); free(s->jobs[t]);
		}
	for (int i = 0; i < s->nworkers; i++) cudaStreamDestroy(s->streams[i]);
	free(s->jobs); free(s->th); free(s->streams);
	pthread_mutex_destroy(&s->mu);
	pthread_cond_destroy(&s->cv_work);
	pthread_cond_destroy(&s->cv_done);
	free(s);
}
