/*
 * yaff_oracle_mt.c -- the oracle's force evaluation spread over host threads.
 *
 * TEST AND BASELINE INFRASTRUCTURE ONLY.  The reference evaluates a force
 * field on one thread; this file runs the same algorithm (the single-thread
 * oracle of yaff_oracle.c, included below, which restates yaff/pes/*.c) on
 * all host cores so that one whole ForceField.compute of a benchmark-sized
 * system can be timed in seconds instead of minutes.  Work is split without
 * changing what is computed:
 *
 *   - neighbour list: the reference's outer atom loop (yaff/pes/nlist.c:55)
 *     is cut into consecutive ranges, each built into a private buffer, and
 *     the buffers are concatenated in order -- the rows are identical to the
 *     single-thread list, in the same order;
 *   - pair terms: consecutive row ranges, private gradient and virial
 *     arrays, summed in range order (yaff/pes/pair_pot.c:84-176 per range);
 *   - Ewald reciprocal sum: consecutive ranges of the half-sphere k-vectors,
 *     private work / gradient / virial arrays, summed in range order, then
 *     the reference's finishing steps (yaff/pes/ewald.c:137-150).
 *
 * Energies, gradients and virials therefore differ from the single-thread
 * oracle only by the order of the final sums (rounding), and the list is
 * bit-identical.  Threads take ranges from a shared counter.
 */
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#include "yaff_oracle.c"

typedef struct {
  void (*run)(void *job, int64_t item);
  void *job;
  int64_t nitem;
  int64_t next;
  pthread_mutex_t lock;
} orc_pool;

static void *orc_pool_worker(void *arg) {
  orc_pool *p = (orc_pool *)arg;
  for (;;) {
    int64_t it;
    pthread_mutex_lock(&p->lock);
    it = p->next++;
    pthread_mutex_unlock(&p->lock);
    if (it >= p->nitem) return NULL;
    p->run(p->job, it);
  }
}

/* Runs run(job, i) for i in [0, nitem) on nthreads threads (the caller's
 * thread is one of them). */
static void orc_parallel(void (*run)(void *, int64_t), void *job, int64_t nitem, int nthreads) {
  orc_pool p;
  pthread_t *tid;
  char *ok;
  int t;
  p.run = run;
  p.job = job;
  p.nitem = nitem;
  p.next = 0;
  pthread_mutex_init(&p.lock, NULL);
  if (nthreads < 1) nthreads = 1;
  tid = (pthread_t *)malloc(sizeof(pthread_t) * (size_t)nthreads);
  ok = (char *)calloc((size_t)nthreads, 1);
  /* a thread that cannot be started leaves its share to the others */
  for (t = 1; t < nthreads && tid && ok; t++) ok[t] = pthread_create(&tid[t], NULL, orc_pool_worker, &p) == 0;
  orc_pool_worker(&p);
  for (t = 1; t < nthreads && tid && ok; t++)
    if (ok[t]) pthread_join(tid[t], NULL);
  free(tid);
  free(ok);
  pthread_mutex_destroy(&p.lock);
}

/* ----------------------------------------------------------- nlist -- */

typedef struct {
  const double *pos;
  int64_t natom, nlow, nhigh;
  double rcut;
  const int64_t *rmax;
  const double *rv, *gv;
  int nvec;
  int64_t *bounds;    /* nrange + 1 atom indices */
  orc_neigh **rows;   /* per range */
  int64_t *cap, *count;
  int failed;
} orc_nl_job;

static void orc_nl_range(void *arg, int64_t r) {
  orc_nl_job *j = (orc_nl_job *)arg;
  for (;;) {
    int64_t n = orc_nlist_build_range(j->pos, j->natom, j->rcut, j->rmax, j->rv, j->gv, j->nvec, j->nlow, j->nhigh,
                                      j->bounds[r], j->bounds[r + 1], j->rows[r], j->cap[r]);
    if (n <= j->cap[r]) {
      j->count[r] = n;
      return;
    }
    free(j->rows[r]);
    j->cap[r] = n + n / 8 + 64;
    j->rows[r] = (orc_neigh *)malloc(sizeof(orc_neigh) * (size_t)j->cap[r]);
    if (!j->rows[r]) {
      j->failed = 1;
      j->count[r] = 0;
      return;
    }
  }
}

/* orc_nlist_build on nthreads threads: the same rows in the same order.
 * rows_hint is the expected row count (the previous list's), used to size the
 * private buffers.  Returns the total row count (rows beyond cap are not
 * written) or -1 when a private buffer could not be allocated. */
int64_t orc_mt_nlist_build(const double *pos, int64_t natom, double rcut, const int64_t *rmax, const double *rv,
                           const double *gv, int nvec, int64_t nlow, int64_t nhigh, orc_neigh *out, int64_t cap,
                           int64_t rows_hint, int nthreads) {
  orc_nl_job j;
  int64_t nrange = 8 * (int64_t)(nthreads > 0 ? nthreads : 1), r, total = 0;
  if (natom - nlow < nrange) nrange = natom - nlow > 0 ? natom - nlow : 1;
  memset(&j, 0, sizeof(j));
  j.pos = pos; j.natom = natom; j.nlow = nlow; j.nhigh = nhigh; j.rcut = rcut; j.rmax = rmax;
  j.rv = rv; j.gv = gv; j.nvec = nvec;
  j.bounds = (int64_t *)malloc(sizeof(int64_t) * (size_t)(nrange + 1));
  j.rows = (orc_neigh **)calloc((size_t)nrange, sizeof(orc_neigh *));
  j.cap = (int64_t *)calloc((size_t)nrange, sizeof(int64_t));
  j.count = (int64_t *)calloc((size_t)nrange, sizeof(int64_t));
  /* the inner loop runs over b <= a, so equal work puts the range bounds at
   * sqrt-spaced atom indices (measured from atom 0) */
  for (r = 0; r <= nrange; r++) {
    double a0 = (double)nlow, a1 = (double)natom;
    double f = sqrt(a0 * a0 + (a1 * a1 - a0 * a0) * (double)r / (double)nrange);
    int64_t b = (int64_t)f;
    if (b < nlow) b = nlow;
    if (b > natom) b = natom;
    if (r == nrange) b = natom;
    if (r > 0 && b < j.bounds[r - 1]) b = j.bounds[r - 1];
    j.bounds[r] = b;
  }
  for (r = 0; r < nrange; r++) {
    double w0 = (double)j.bounds[r], w1 = (double)j.bounds[r + 1];
    double share = (w1 * w1 - w0 * w0) / ((double)natom * natom - (double)nlow * nlow + 1.0);
    j.cap[r] = (int64_t)(1.2 * share * (double)rows_hint) + 1024;
    j.rows[r] = (orc_neigh *)malloc(sizeof(orc_neigh) * (size_t)j.cap[r]);
    if (!j.rows[r]) j.failed = 1;
  }
  if (!j.failed) orc_parallel(orc_nl_range, &j, nrange, nthreads);
  for (r = 0; r < nrange; r++) {
    if (!j.failed) {
      int64_t take = j.count[r];
      if (total < cap) {
        int64_t room = cap - total;
        memcpy(out + total, j.rows[r], sizeof(orc_neigh) * (size_t)(take < room ? take : room));
      }
      total += take;
    }
    free(j.rows[r]);
  }
  free(j.bounds); free(j.rows); free(j.cap); free(j.count);
  return j.failed ? -1 : total;
}

/* ------------------------------------------------------------ pairs -- */

typedef struct {
  const orc_neigh *rows;
  int64_t n, nst, natom, nrange;
  const orc_scale *st;
  orc_pairpot pp;
  double *gpos, *vtens, *energy;   /* per range: natom*3, 9, 1 (gpos/vtens may be NULL) */
  int want_g, want_v;
} orc_pair_job;

static void orc_pair_range(void *arg, int64_t r) {
  orc_pair_job *j = (orc_pair_job *)arg;
  int64_t i0 = j->n * r / j->nrange, i1 = j->n * (r + 1) / j->nrange;
  j->energy[r] = orc_pair_loop(j->rows + i0, i1 - i0, j->st, j->nst, &j->pp,
                               j->want_g ? j->gpos + (size_t)r * 3 * j->natom : NULL,
                               j->want_v ? j->vtens + 9 * r : NULL);
}

/* orc_pair_compute on nthreads threads (natom sizes the private gradients). */
double orc_mt_pair_compute(const orc_neigh *rows, int64_t n, const orc_scale *st, int64_t nst, int kind,
                           const double *sigma, const double *epsilon, const int32_t *onlypauli,
                           const double *charges, const double *radii, double alpha, double dielectric, double rcut,
                           int tr_kind, double tr_par, double *gpos, double *vtens, int64_t natom, int nthreads) {
  orc_pair_job j;
  int64_t r, i;
  double e = 0.0;
  memset(&j, 0, sizeof(j));
  j.rows = rows; j.n = n; j.st = st; j.nst = nst; j.natom = natom;
  j.nrange = 4 * (int64_t)(nthreads > 0 ? nthreads : 1);
  j.pp.kind = kind; j.pp.sigma = sigma; j.pp.epsilon = epsilon; j.pp.onlypauli = onlypauli;
  j.pp.charges = charges; j.pp.radii = radii; j.pp.alpha = alpha; j.pp.dielectric = dielectric;
  j.pp.rcut = rcut; j.pp.tr_kind = tr_kind; j.pp.tr_par = tr_par;
  j.want_g = gpos != NULL;
  j.want_v = vtens != NULL;
  j.energy = (double *)calloc((size_t)j.nrange, sizeof(double));
  if (j.want_g) j.gpos = (double *)calloc((size_t)(j.nrange * 3 * natom), sizeof(double));
  if (j.want_v) j.vtens = (double *)calloc((size_t)(j.nrange * 9), sizeof(double));
  if (!j.energy || (j.want_g && !j.gpos) || (j.want_v && !j.vtens)) {
    free(j.energy); free(j.gpos); free(j.vtens);
    return NAN;
  }
  orc_parallel(orc_pair_range, &j, j.nrange, nthreads);
  for (r = 0; r < j.nrange; r++) {
    e += j.energy[r];
    if (j.want_g)
      for (i = 0; i < 3 * natom; i++) gpos[i] += j.gpos[(size_t)r * 3 * natom + i];
    if (j.want_v)
      for (i = 0; i < 9; i++) vtens[i] += j.vtens[9 * r + i];
  }
  free(j.energy); free(j.gpos); free(j.vtens);
  return e;
}

/* ------------------------------------------------------------ Ewald -- */

typedef struct {
  const double *pos, *charges, *gv;
  int64_t natom, nlow, nhigh, nk, nrange;
  double volume, alpha, gcut;
  const int64_t *gmax;
  double *gpos, *work, *vtens, *energy;
  int want_g, want_v;
} orc_ew_job;

static void orc_ew_range(void *arg, int64_t r) {
  orc_ew_job *j = (orc_ew_job *)arg;
  int64_t k0 = j->nk * r / j->nrange, k1 = j->nk * (r + 1) / j->nrange;
  j->energy[r] = orc_ewald_reci_range(j->pos, j->natom, j->nlow, j->nhigh, j->charges, j->gv, j->volume, j->alpha,
                                      j->gmax, j->gcut, k0, k1,
                                      j->want_g ? j->gpos + (size_t)r * 3 * j->natom : NULL,
                                      j->want_g ? j->work + (size_t)r * 2 * j->natom : NULL,
                                      j->want_v ? j->vtens + 9 * r : NULL);
}

/* orc_ewald_reci on nthreads threads. */
double orc_mt_ewald_reci(const double *pos, int64_t natom, int64_t nlow, int64_t nhigh, const double *charges,
                         const double *rv, const double *gv, double volume, double alpha, const int64_t *gmax,
                         double gcut, double dielectric, double *gpos, double *vtens, int nthreads) {
  orc_ew_job j;
  int64_t g0, g1, g2, r, i, nk = 0;
  double energy = 0.0, kv[9], gc2, dfac;
  (void)rv;
  for (i = 0; i < 9; i++) kv[i] = ORC_TWO_PI * gv[i];
  gc2 = gcut * ORC_TWO_PI;
  gc2 *= gc2;
  for (g0 = -gmax[0]; g0 <= gmax[0]; g0++)
    for (g1 = -gmax[1]; g1 <= gmax[1]; g1++)
      for (g2 = 0; g2 <= gmax[2]; g2++) {
        double k[3];
        if (g2 == 0 && (g1 < 0 || (g1 == 0 && g0 <= 0))) continue;
        k[0] = (g0 * kv[0] + g1 * kv[3] + g2 * kv[6]);
        k[1] = (g0 * kv[1] + g1 * kv[4] + g2 * kv[7]);
        k[2] = (g0 * kv[2] + g1 * kv[5] + g2 * kv[8]);
        if (k[0] * k[0] + k[1] * k[1] + k[2] * k[2] <= gc2) nk++;
      }
  memset(&j, 0, sizeof(j));
  j.pos = pos; j.charges = charges; j.gv = gv; j.natom = natom; j.nlow = nlow; j.nhigh = nhigh; j.nk = nk;
  j.volume = volume; j.alpha = alpha; j.gcut = gcut; j.gmax = gmax;
  j.nrange = 4 * (int64_t)(nthreads > 0 ? nthreads : 1);
  if (j.nrange > nk) j.nrange = nk > 0 ? nk : 1;
  j.want_g = gpos != NULL;
  j.want_v = vtens != NULL;
  j.energy = (double *)calloc((size_t)j.nrange, sizeof(double));
  if (j.want_g) {
    j.gpos = (double *)calloc((size_t)(j.nrange * 3 * natom), sizeof(double));
    j.work = (double *)calloc((size_t)(j.nrange * 2 * natom), sizeof(double));
  }
  if (j.want_v) j.vtens = (double *)calloc((size_t)(j.nrange * 9), sizeof(double));
  if (!j.energy || (j.want_g && (!j.gpos || !j.work)) || (j.want_v && !j.vtens)) {
    free(j.energy); free(j.gpos); free(j.work); free(j.vtens);
    return NAN;
  }
  orc_parallel(orc_ew_range, &j, j.nrange, nthreads);
  for (r = 0; r < j.nrange; r++) {
    energy += j.energy[r];
    if (j.want_g)
      for (i = 0; i < 3 * natom; i++) gpos[i] += j.gpos[(size_t)r * 3 * natom + i];
    if (j.want_v)
      for (i = 0; i < 9; i++) vtens[i] += j.vtens[9 * r + i];
  }
  free(j.energy); free(j.gpos); free(j.work); free(j.vtens);
  if (vtens) { vtens[0] -= energy; vtens[4] -= energy; vtens[8] -= energy; }
  dfac = 1.0 / dielectric;
  if (gpos) for (i = 0; i < 3 * natom; i++) gpos[i] *= dfac;
  if (vtens) for (i = 0; i < 9; i++) vtens[i] *= dfac;
  return energy * dfac;
}
