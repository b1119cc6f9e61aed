// yg_mc.cu -- Monte Carlo trial energies on the GPU.
//
// The reference evaluates one trial move of a rigid guest at a time
// (yaff/sampling/mctrials.py:69-126): a full force-field evaluation of the
// guest against everything else (neighbour list filtered to guest-other pairs
// by nlow = nhigh, nlist.c:57; LJ and the real-space Ewald term) and the
// reciprocal-space interaction through structure factors
// (ForcePartEwaldReciprocalInteraction, yaff/pes/ff.py:1060-1255, on
// compute_ewald_prefactors / structurefactors / deltae, ewald.c:441-522).
// Here a batch of trials -- insertions, deletions and translations of many
// chains -- is one launch: one thread block per trial sums the guest-other
// pair terms over the framework and the chain's other guests and the
// reciprocal interaction over the k vectors of the half sphere against the
// chain's resident structure factors.  Accepted moves update the resident
// positions and structure factors in place (mctrials.py:177-190).
//
// Structure factors live on a compact list of the k vectors inside the
// cutoff, in the reference's loop order; the reference's dense arrays
// ((2 gmax0+1) x (2 gmax1+1) x (gmax2+1), with the element of each k stored
// one position after its loop index, ewald.c:457/488) are produced only at
// the API boundary.
#include <cmath>
#include <cstring>
#include <vector>

#include "yg_internal.cuh"
#include "yg_pairterm.cuh"

#define MC_MAXG 4          // atoms per guest (rigid 3- and 4-site molecules)
#define MC_TB 256          // threads per trial block
#define MC_SF_CHUNK 128    // atoms per structure-factor partial
#define MC_GT 24           // phase-table entries per axis (gmax <= 23)

enum { MC_INSERT = 0, MC_DELETE = 1, MC_TRANSLATE = 2 };

struct yg_mc {
  int precision = YG_FP64;
  cudaStream_t stream = 0;
  CellGeom cell{};
  int rmax[3] = {0, 0, 0};
  double rcut = 0.0, alpha = 0.0, gcut = 0.0, diel = 1.0;
  double close_contact = -1.0;
  int64_t gmax[3] = {0, 0, 0};
  int nk = 0;                      // k vectors inside the cutoff
  std::vector<int64_t> kidx;       // their element in the reference's dense layout
  std::vector<double> pref_dense;  // the reference's prefactor array (+1 element)
  double4_32a *d_k = nullptr;          // kx, ky, kz, prefactor
  int4 *d_kg = nullptr;                // g0, g1, g2 of each k
  int64_t nframe = 0;
  double *d_fpos = nullptr, *d_ffrac = nullptr;
  unsigned *d_ffix = nullptr, *d_gfix = nullptr;  // fixed-point fractions
  int4 *d_cols = nullptr;          // k columns: g0, g1, first g2, first k (+ sentinel)
  int ncol = 0;
  double4_32a *d_fpar = nullptr;       // q, sigma, sqrt(eps)
  float4 *d_fparf = nullptr;           // the same in FP32
  int M = 0;
  double gq[MC_MAXG], gsig[MC_MAXG], gseps[MC_MAXG];
  int64_t nchain = 0, max_guests = 0;
  double *d_gpos = nullptr, *d_gfrac = nullptr;
  int *d_nguest = nullptr;
  std::vector<int> nguest;
  double2 *d_S = nullptr;          // [chain][k]
  float4 *d_Sff = nullptr;         // [chain][k] S as FP32 hi + lo (re hi, im hi, re lo, im lo), mixed trials
  float2 *d_kpf = nullptr;         // [k] prefactor as FP32 hi + lo
  double2 *d_Sframe = nullptr;     // [k]
  double2 *d_Spart = nullptr;      // structure-factor partials
  size_t spart_cap = 0;
  // last trial batch
  int64_t cap_trials = 0, ntrial = 0;
  int4 *d_trials = nullptr;
  double *d_newpos = nullptr, *d_energy = nullptr;
  std::vector<int4> h_trials;
  std::vector<double> h_newpos;
  int64_t launches = 0;
};

namespace {

struct McDev {
  CellGeom cell;
  int rmax[3];
  float rvf[9];
  double rc2;
  float rc2f;
  double alpha, inv_diel;
  float alphaf, inv_dielf;
  double close2;      // close-contact distance squared (negative: off)
  float near2f, rc2f_lo, rc2f_hi;  // mixed: FP64 below near2f and inside (rc2f_lo, rc2f_hi)
  int gmax[3];
  const int4 *kg;     // (g0, g1, g2) of each k
  int nk;
  const double4_32a *k;
  int64_t nframe;
  const double *fpos, *ffrac;
  const unsigned *ffix, *gfix;
  const int4 *cols;
  int ncol;
  const double4_32a *fpar;
  int M;
  double gq[MC_MAXG], gsig[MC_MAXG], gseps[MC_MAXG];
  double gpar[MC_MAXG][3];         // q, sigma, sqrt(eps) per guest atom
  float gqf[MC_MAXG], gsigf[MC_MAXG], gsepsf[MC_MAXG];
  const float4 *fparf;             // framework q, sigma, sqrt(eps) in FP32
  int64_t max_guests;
  const double *gpos, *gfrac;
  const int *nguest;
  const double2 *S;
  const float4 *Sff;               // mixed: S split into FP32 hi + lo per launch
  const float2 *kpf;               // mixed: prefactors as FP32 hi + lo
  float gqh[MC_MAXG], gql[MC_MAXG];  // guest charges as FP32 hi + lo
};

// s - floor(s) as a 32-bit fixed-point fraction: differences of two such
// values, read as int32, are the minimum-image fractional difference with
// the wrap done exactly by integer arithmetic.
__device__ __forceinline__ unsigned mc_fix(double s) {
  const double w = s - floor(s);
  return (unsigned)((unsigned long long)(w * 4294967296.0) & 0xffffffffull);
}

// Fractional coordinates s = G r (FP64) and their fixed-point form (for
// the mixed path).
__global__ void k_mc_frac(const double *__restrict__ pos, int64_t n, CellGeom cell, double *__restrict__ frac,
                          unsigned *__restrict__ fix) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double x = pos[3 * i], y = pos[3 * i + 1], z = pos[3 * i + 2];
#pragma unroll
  for (int a = 0; a < 3; a++) {
    const double f = cell.gv[3 * a] * x + cell.gv[3 * a + 1] * y + cell.gv[3 * a + 2] * z;
    frac[3 * i + a] = f;
    fix[3 * i + a] = mc_fix(f);
  }
}

// Partial structure factors: part[chunk][k] = sum over the chunk's atoms of
// q (cos kr, sin kr), x = k0 x + k1 y + k2 z in the reference's order
// (ewald.c:500-503).  Charges per atom (q) or from the guest template
// (q == nullptr: charge of atom i is tq[i % M]).
__global__ void k_mc_sfac_part(const double4_32a *__restrict__ kv, int nk, const double *__restrict__ pos,
                               const double *__restrict__ q, const McDev D, int64_t natom,
                               double2 *__restrict__ part) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int64_t a0 = (int64_t)blockIdx.y * MC_SF_CHUNK;
  if (k >= nk) return;
  const double4_32a K = kv[k];
  double c = 0.0, s = 0.0;
  const int64_t a1 = min(natom, a0 + MC_SF_CHUNK);
  for (int64_t i = a0; i < a1; i++) {
    const double x = xadd(xadd(xmul(K.x, pos[3 * i]), xmul(K.y, pos[3 * i + 1])), xmul(K.z, pos[3 * i + 2]));
    const double qi = q ? q[i] : D.gq[i % D.M];
    double sn, cs;
    sincos(x, &sn, &cs);
    c = xadd(c, xmul(qi, cs));
    s = xadd(s, xmul(qi, sn));
  }
  part[(int64_t)blockIdx.y * nk + k] = make_double2(c, s);
}

// out[k] (+)= sum of the partials in chunk order
__global__ void k_mc_sfac_sum(const double2 *__restrict__ part, int nchunk, int nk, const double2 *__restrict__ base,
                              double2 *__restrict__ out) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  if (k >= nk) return;
  double c = 0.0, s = 0.0;
  for (int ch = 0; ch < nchunk; ch++) {
    const double2 v = part[(int64_t)ch * nk + k];
    c += v.x;
    s += v.y;
  }
  if (base) {
    c = base[k].x + c;
    s = base[k].y + s;
  }
  out[k] = make_double2(c, s);
}

// Energy sum of one side of a trial (guest vs framework, or guest vs the
// other guests): FP64, or an FP32 TwoSum pair; plus the smallest MIC
// distance squared for the close-contact rule.
struct McSum {
  double e64;
  float eh, el;
  double dmin2;    // FP64 path
  float dmin2f;    // mixed path
  __device__ __forceinline__ void init() {
    e64 = 0.0;
    eh = 0.f;
    el = 0.f;
    dmin2 = 1e300;
    dmin2f = 3.0e38f;
  }
  __device__ __forceinline__ void add32(float v) {
    const float sum = eh + v, bb = sum - eh;
    el += (eh - (sum - bb)) + (v - bb);
    eh = sum;
  }
  __device__ __forceinline__ double value() const { return e64 + ((double)eh + (double)el); }
};

__device__ __forceinline__ void mc_terms64(const McDev &D, double dd, double d2, double qa, double sa, double ea,
                                           double qj, double sj, double ej, McSum &acc) {
  PairPotDev lj, ei;
  lj.kind = YG_POT_LJ;
  lj.tr_kind = YG_TR_NONE;
  ei.kind = YG_POT_EI;
  ei.tr_kind = YG_TR_NONE;
  double v, g;
  pair_term<double>(lj, 0.0, 0.0, 0.0, 1.0, dd, d2, sa, ea, 0.0, 0.0, sj, ej, 0.0, 0.0, 0.0, 0.0, v, g);
  acc.e64 += v;
  pair_term<double>(ei, 0.0, 0.0, D.alpha, D.inv_diel, dd, d2, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, 0.0, qa, qj, v, g);
  acc.e64 += v;
}

// One (guest atom, other atom) pair, all images within the cutoff: LJ +
// real-space EI into acc, FP64 with the reference's relative vector (other -
// guest, sequential wrap, image vectors added axis by axis; nlist.c:57-95).
__device__ __forceinline__ void mc_pair64(const McDev &D, const double *ga, double qa, double sa, double ea,
                                          const double *pj, double qj, double sj, double ej, McSum &acc) {
  double d0[3] = {xsub(pj[0], ga[0]), xsub(pj[1], ga[1]), xsub(pj[2], ga[2])};
  int m[3];
  exact_mic(d0, D.cell, m);
  acc.dmin2 = fmin(acc.dmin2, exact_norm2(d0));
  for (int r0 = -D.rmax[0]; r0 <= D.rmax[0]; r0++)
    for (int r1 = -D.rmax[1]; r1 <= D.rmax[1]; r1++)
      for (int r2 = -D.rmax[2]; r2 <= D.rmax[2]; r2++) {
        double d[3] = {d0[0], d0[1], d0[2]};
        const int img[3] = {r0, r1, r2};
        if (r0 | r1 | r2) exact_add_vec(d, D.cell, img);
        const double d2 = exact_norm2(d);
        if (!(d2 < D.rc2)) continue;
        mc_terms64(D, sqrt(d2), d2, qa, sa, ea, qj, sj, ej, acc);
      }
}

// The same pair, mixed: the minimum-image fractional difference from the
// 32-bit fixed-point fractions (exact integer wrap), FP32 Cartesian vector
// and terms.  Pairs closer than D.near (where the terms are large:
// erfc(alpha d) > 5e-3) or within 1e-6 of the cutoff are not evaluated here:
// they go to the warp's queue of deferred pairs (ballot-compacted, so that
// the FP64 terms later run on full warps instead of on the few lanes of a
// warp that meet such a pair) and are recomputed in FP64 from the FP64
// fractions on the same image, so the energy difference keeps ~1e-9 Ha
// absolute accuracy.  All lanes of the warp call this together (valid marks
// the lanes with a real pair); code = guest atom | side << 2.
#define MC_QCAP 64  // deferred pairs per warp (a flush at 32 leaves at most 31)

struct McDefer {
  int j;         // other atom: framework index (sides 0, 2) or guest-slot index u (sides 1, 3)
  int code;      // guest atom | side << 2 | (r0 + 8) << 4 | (r1 + 8) << 9 | (r2 + 8) << 14
};

template <typename Drain>
__device__ __forceinline__ void mc_pair32(const McDev &D, const unsigned *xa, float qa, float sa, float ea,
                                          const unsigned *xj, float qj, float sj, float ej, bool valid, int j,
                                          int code, McSum &acc, McDefer *wq, int &qn, unsigned lt, Drain &drain) {
  int di[3];
  float sfr[3];
#pragma unroll
  for (int x = 0; x < 3; x++) {
    di[x] = valid ? (int)(xj[x] - xa[x]) : 0;
    sfr[x] = (float)di[x] * 2.3283064365386963e-10f;  // 2^-32
  }
  float d0[3];
#pragma unroll
  for (int x = 0; x < 3; x++) d0[x] = sfr[0] * D.rvf[x] + sfr[1] * D.rvf[3 + x] + sfr[2] * D.rvf[6 + x];
  if (valid) acc.dmin2f = fminf(acc.dmin2f, d0[0] * d0[0] + d0[1] * d0[1] + d0[2] * d0[2]);
  for (int r0 = -D.rmax[0]; r0 <= D.rmax[0]; r0++)
    for (int r1 = -D.rmax[1]; r1 <= D.rmax[1]; r1++)
      for (int r2 = -D.rmax[2]; r2 <= D.rmax[2]; r2++) {
        float d[3];
#pragma unroll
        for (int x = 0; x < 3; x++)
          d[x] = d0[x] + (float)r0 * D.rvf[x] + (float)r1 * D.rvf[3 + x] + (float)r2 * D.rvf[6 + x];
        const float d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
        const bool in = valid && d2 < D.rc2f_hi;
        const bool defer = in && (d2 < D.near2f || d2 > D.rc2f_lo);
        if (in && !defer) {
          PairPotDev lj, ei;
          lj.kind = YG_POT_LJ;
          lj.tr_kind = YG_TR_NONE;
          ei.kind = YG_POT_EI;
          ei.tr_kind = YG_TR_NONE;
          const float inv_d = rsqrtf(d2);
          const float dd = d2 * inv_d;
          float v, g, v2;
          pair_term_f32(lj, 0.f, 0.f, 0.f, 1.f, dd, d2, inv_d, sa, ea, 0.f, 0.f, sj, ej, 0.f, 0.f, 0.f, 0.f, v, g);
          pair_term_f32(ei, 0.f, 0.f, D.alphaf, D.inv_dielf, dd, d2, inv_d, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f, 0.f,
                        qa, qj, v2, g);
          acc.add32(v + v2);
        }
        const unsigned b = __ballot_sync(0xffffffffu, defer);
        if (defer) {
          McDefer e;
          e.j = j;
          e.code = code | ((r0 + 8) << 4) | ((r1 + 8) << 9) | ((r2 + 8) << 14);
          wq[qn + __popc(b & lt)] = e;
        }
        qn += __popc(b);
        drain(false);  // at most 31 left: the next image's pairs fit
      }
}

// FP64 terms of deferred pairs 0 .. n-1 of the warp's queue, one per lane;
// the energies go to e[side].
__device__ __forceinline__ void mc_flush(const McDev &D, const McDefer *wq, int n, int lane, int64_t gbase,
                                         const double *fold, const double *fnew, const unsigned *xold,
                                         const unsigned *xnew, double (&e)[4]) {
  if (lane >= n) return;
  const McDefer q = wq[lane];
  const int a = q.code & 3, side = (q.code >> 2) & 3;
  const int r[3] = {((q.code >> 4) & 31) - 8, ((q.code >> 9) & 31) - 8, ((q.code >> 14) & 31) - 8};
  const double *fa = ((side & 2) ? fnew : fold) + 3 * a;
  const unsigned *xa = ((side & 2) ? xnew : xold) + 3 * a;
  const double *fj, *pj;
  const unsigned *xj;
  if (side & 1) {
    fj = D.gfrac + (gbase + q.j) * 3;
    xj = D.gfix + (gbase + q.j) * 3;
    pj = D.gpar[q.j % D.M];
  } else {
    fj = D.ffrac + 3 * (int64_t)q.j;
    xj = D.ffix + 3 * (int64_t)q.j;
    pj = (const double *)(D.fpar + q.j);
  }
  // FP64 fractional difference on the image the fixed-point wrap chose
  double u[3];
#pragma unroll
  for (int x = 0; x < 3; x++) {
    const double t = fj[x] - fa[x];
    u[x] = t - rint(t - (double)(int)(xj[x] - xa[x]) * 2.3283064365386963e-10) + r[x];
  }
  double c[3];
#pragma unroll
  for (int x = 0; x < 3; x++) c[x] = u[0] * D.cell.rv[x] + u[1] * D.cell.rv[3 + x] + u[2] * D.cell.rv[6 + x];
  const double d2d = c[0] * c[0] + c[1] * c[1] + c[2] * c[2];
  if (!(d2d < D.rc2)) return;
  McSum tmp;
  tmp.init();
  const double *pa = D.gpar[a];
  mc_terms64(D, sqrt(d2d), d2d, pa[0], pa[1], pa[2], pj[0], pj[1], pj[2], tmp);
  e[side] += tmp.e64;
}

// Double-float arithmetic (a value as an unevaluated FP32 sum hi + lo, about
// 44 significant bits): the mixed trials' reciprocal sum runs on the FP32
// pipe with close to FP64 accuracy.  The _rn intrinsics keep the compiler
// from fusing the error-free steps.
struct McFF {
  float h, l;
};
__device__ __forceinline__ McFF ff_mul(McFF a, McFF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  const float s = __fadd_rn(p, e);
  return McFF{s, __fsub_rn(e, __fsub_rn(s, p))};
}
__device__ __forceinline__ McFF ff_add(McFF a, McFF b) {
  const float s = __fadd_rn(a.h, b.h);
  const float bb = __fsub_rn(s, a.h);
  float t = __fadd_rn(__fsub_rn(a.h, __fsub_rn(s, bb)), __fsub_rn(b.h, bb));
  t = __fadd_rn(t, __fadd_rn(a.l, b.l));
  const float r = __fadd_rn(s, t);
  return McFF{r, __fsub_rn(t, __fsub_rn(r, s))};
}
__device__ __forceinline__ McFF ff_neg(McFF a) { return McFF{-a.h, -a.l}; }
// acc += a b, acc left unnormalized (hi exact TwoSum, errors gathered in lo)
__device__ __forceinline__ void ff_acc(McFF &acc, McFF a, McFF b) {
  const float p = __fmul_rn(a.h, b.h);
  float e = fmaf(a.h, b.h, -p);
  e = fmaf(a.h, b.l, e);
  e = fmaf(a.l, b.h, e);
  const float s = __fadd_rn(acc.h, p);
  const float bb = __fsub_rn(s, acc.h);
  const float t = __fadd_rn(__fsub_rn(acc.h, __fsub_rn(s, bb)), __fsub_rn(p, bb));
  acc.h = s;
  acc.l = __fadd_rn(acc.l, __fadd_rn(t, e));
}

// The chains' structure factors as FP32 hi + lo, once per trial launch.
__global__ void k_mc_split_s(const double2 *__restrict__ S, int64_t n, float4 *__restrict__ out) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= n) return;
  const double2 v = S[i];
  const float xh = (float)v.x, yh = (float)v.y;
  out[i] = make_float4(xh, yh, (float)(v.x - (double)xh), (float)(v.y - (double)yh));
}

// q (cos x, sin x) of one atom for one k: FP64 (the reference's op order)
// or, mixed, an FP64 phase reduced exactly to [-pi, pi] and FP32 sincos.
template <bool F64>
__device__ __forceinline__ void mc_phase(const double4_32a &K, const double *p, double q, double &c, double &s) {
  const double x = xadd(xadd(xmul(K.x, p[0]), xmul(K.y, p[1])), xmul(K.z, p[2]));
  if (F64) {
    double sn, cs;
    sincos(x, &sn, &cs);
    c = q * cs;
    s = q * sn;
  } else {
    const double two_pi = 6.283185307179586476925;
    const double r = x - two_pi * rint(x * (1.0 / two_pi));
    float sn, cs;
    sincosf((float)r, &sn, &cs);
    c = q * (double)cs;
    s = q * (double)sn;
  }
}

// One block per trial: E = -(E_old + R_old) [delete, translate]
//                          +(E_new + R_new) [insert, translate]
// E_* = guest-framework + guest-other-guests energy (LJ + real-space EI),
// each side replaced by 1e10 when the guest comes closer than the
// close-contact distance to an atom of that side (mctrials.py:75-111);
// R_old = 2 sum pref (S - dS_old).dS_old, R_new = 2 sum pref (S - [translate]
// dS_old).dS_new, over eps_r (ff.py:1211-1253, ewald.c:508-522).
template <bool F64>
__global__ void __launch_bounds__(MC_TB, 1) k_mc_trials(const McDev D, const int4 *__restrict__ trials,
                                                    const double *__restrict__ newpos, double *__restrict__ energy) {
  __shared__ double sh_old[MC_MAXG * 3], sh_new[MC_MAXG * 3], sh_fold[MC_MAXG * 3], sh_fnew[MC_MAXG * 3];
  __shared__ unsigned sh_xold[MC_MAXG * 3], sh_xnew[MC_MAXG * 3];
  __shared__ double red[MC_TB / 32][10];
  __shared__ double2 sh_tab[2 * MC_MAXG][3][MC_GT];
  __shared__ McDefer sh_q[MC_TB / 32][MC_QCAP];
  __shared__ float4 sh_tabf[F64 ? 1 : 2 * MC_MAXG][3][MC_GT];
  const int t = blockIdx.x;
  const int4 tr = trials[t];
  const int chain = tr.x, kind = tr.y, guest = tr.z;
  const int M = D.M;
  const bool has_old = kind != MC_INSERT, has_new = kind != MC_DELETE;
  const int64_t gbase = ((int64_t)chain * D.max_guests) * M;
  if (threadIdx.x < 3 * M) {
    const int i = threadIdx.x;
    if (has_old) {
      sh_old[i] = D.gpos[(gbase + (int64_t)guest * M) * 3 + i];
      sh_fold[i] = D.gfrac[(gbase + (int64_t)guest * M) * 3 + i];
      sh_xold[i] = D.gfix[(gbase + (int64_t)guest * M) * 3 + i];
    }
    if (has_new) sh_new[i] = newpos[(int64_t)t * M * 3 + i];
  }
  __syncthreads();
  if (has_new && threadIdx.x < M) {
    const double *p = sh_new + 3 * threadIdx.x;
#pragma unroll
    for (int a = 0; a < 3; a++) {
      const double f = D.cell.gv[3 * a] * p[0] + D.cell.gv[3 * a + 1] * p[1] + D.cell.gv[3 * a + 2] * p[2];
      sh_fnew[3 * threadIdx.x + a] = f;
      sh_xnew[3 * threadIdx.x + a] = mc_fix(f);
    }
  }
  __syncthreads();
  // real space: [0] old vs framework, [1] old vs guests, [2] new vs
  // framework, [3] new vs guests
  McSum acc[4];
#pragma unroll
  for (int q = 0; q < 4; q++) acc[q].init();
  const int ng = D.nguest[chain];
  if (F64) {
    for (int64_t j = threadIdx.x; j < D.nframe; j += MC_TB) {
      const double4_32a pr = D.fpar[j];
      for (int a = 0; a < M; a++) {
        if (has_old) mc_pair64(D, sh_old + 3 * a, D.gq[a], D.gsig[a], D.gseps[a], D.fpos + 3 * j, pr.x, pr.y, pr.z, acc[0]);
        if (has_new) mc_pair64(D, sh_new + 3 * a, D.gq[a], D.gsig[a], D.gseps[a], D.fpos + 3 * j, pr.x, pr.y, pr.z, acc[2]);
      }
    }
    for (int64_t u = threadIdx.x; u < (int64_t)ng * M; u += MC_TB) {
      const int gi = (int)(u / M), ai = (int)(u % M);
      if (has_old && gi == guest) continue;  // the moving guest itself
      const double *pj = D.gpos + (gbase + u) * 3;
      for (int a = 0; a < M; a++) {
        if (has_old) mc_pair64(D, sh_old + 3 * a, D.gq[a], D.gsig[a], D.gseps[a], pj, D.gq[ai], D.gsig[ai], D.gseps[ai], acc[1]);
        if (has_new) mc_pair64(D, sh_new + 3 * a, D.gq[a], D.gsig[a], D.gseps[a], pj, D.gq[ai], D.gsig[ai], D.gseps[ai], acc[3]);
      }
    }
  } else {
    // every lane of a warp takes the same loop trips (valid marks the real
    // pairs): the deferred-pair queue is filled and flushed warp-wide
    McDefer *wq = sh_q[threadIdx.x >> 5];
    const int lane = threadIdx.x & 31;
    const unsigned lt = (1u << lane) - 1u;
    int qn = 0;
    double edef[4] = {0.0, 0.0, 0.0, 0.0};
    auto drain = [&](bool all) {
      while (qn >= 32 || (all && qn > 0)) {
        __syncwarp();
        mc_flush(D, wq, qn < 32 ? qn : 32, lane, gbase, sh_fold, sh_fnew, sh_xold, sh_xnew, edef);
        __syncwarp();
        const int rest = qn > 32 ? qn - 32 : 0;
        McDefer mv;
        if (lane < rest) mv = wq[32 + lane];
        __syncwarp();
        if (lane < rest) wq[lane] = mv;
        __syncwarp();
        qn = rest;
      }
    };
    for (int64_t jb = 0; jb < D.nframe; jb += MC_TB) {
      const int64_t j = jb + threadIdx.x;
      const bool vj = j < D.nframe;
      const float4 pf = vj ? D.fparf[j] : make_float4(0.f, 0.f, 0.f, 0.f);
      const unsigned *xj = D.ffix + 3 * (vj ? j : 0);
      for (int a = 0; a < M; a++) {
        if (has_old) {
          mc_pair32(D, sh_xold + 3 * a, D.gqf[a], D.gsigf[a], D.gsepsf[a], xj, pf.x, pf.y, pf.z, vj, (int)j, a | (0 << 2),
                    acc[0], wq, qn, lt, drain);
        }
        if (has_new) {
          mc_pair32(D, sh_xnew + 3 * a, D.gqf[a], D.gsigf[a], D.gsepsf[a], xj, pf.x, pf.y, pf.z, vj, (int)j, a | (2 << 2),
                    acc[2], wq, qn, lt, drain);
        }
      }
    }
    for (int64_t ub = 0; ub < (int64_t)ng * M; ub += MC_TB) {
      const int64_t u = ub + threadIdx.x;
      const int gi = (int)(u / M), ai = (int)(u % M);
      const bool vu = u < (int64_t)ng * M && !(has_old && gi == guest);  // not the moving guest itself
      const unsigned *xj = D.gfix + (gbase + (vu ? u : 0)) * 3;
      for (int a = 0; a < M; a++) {
        if (has_old) {
          mc_pair32(D, sh_xold + 3 * a, D.gqf[a], D.gsigf[a], D.gsepsf[a], xj, D.gqf[ai], D.gsigf[ai], D.gsepsf[ai],
                    vu, (int)u, a | (1 << 2), acc[1], wq, qn, lt, drain);
        }
        if (has_new) {
          mc_pair32(D, sh_xnew + 3 * a, D.gqf[a], D.gsigf[a], D.gsepsf[a], xj, D.gqf[ai], D.gsigf[ai], D.gsepsf[ai],
                    vu, (int)u, a | (3 << 2), acc[3], wq, qn, lt, drain);
        }
      }
    }
    drain(true);
    for (int q = 0; q < 4; q++) acc[q].e64 += edef[q];
  }
  double ro = 0.0, rn = 0.0;
  if (F64) {
  // reciprocal space: e^{i k.r} = T0[g0] T1[g1] T2[g2] from per-atom FP64
  // tables e^{2 pi i g s} (s = fractional coordinate), conjugated for g < 0
  const int G0 = D.gmax[0], G1 = D.gmax[1], G2 = D.gmax[2];
  const int ntab = 2 * M * (G0 + G1 + G2 + 3);
  for (int i = threadIdx.x; i < ntab; i += MC_TB) {
    const int slot = i / (G0 + G1 + G2 + 3);
    int r = i - slot * (G0 + G1 + G2 + 3);
    int axis = 0;
    if (r > G0) {
      r -= G0 + 1;
      axis = 1;
      if (r > G1) {
        r -= G1 + 1;
        axis = 2;
      }
    }
    const bool is_new = slot >= M;
    if (is_new ? has_new : has_old) {
      const double f = (is_new ? sh_fnew : sh_fold)[3 * (slot % M) + axis];
      double sn, cs;
      sincospi(2.0 * r * f, &sn, &cs);
      sh_tab[slot][axis][r] = make_double2(cs, sn);
    }
  }
  __syncthreads();
  // one (g0, g1) column per thread: P = q T0[g0] T1[g1] per atom, then
  // dS(k) = sum_atoms P T2[g2] along the column's g2 run
  const double2 *S = D.S + (int64_t)chain * D.nk;
  const int sbeg = has_old ? 0 : M, send = has_new ? 2 * M : M;
  for (int col = threadIdx.x; col < D.ncol; col += MC_TB) {
    const int4 cd = D.cols[col];
    const int kend = D.cols[col + 1].w;
    const int a0 = cd.x < 0 ? -cd.x : cd.x, a1 = cd.y < 0 ? -cd.y : cd.y;
    const double s0 = cd.x < 0 ? -1.0 : 1.0, s1 = cd.y < 0 ? -1.0 : 1.0;
    double pr[2 * MC_MAXG], pi[2 * MC_MAXG];
#pragma unroll
    for (int slot = 0; slot < 2 * MC_MAXG; slot++) {
      if (slot < sbeg || slot >= send) continue;
      const double2 e0 = sh_tab[slot][0][a0], e1 = sh_tab[slot][1][a1];
      const double e0i = s0 * e0.y, e1i = s1 * e1.y;
      const double q = D.gq[slot % M];
      pr[slot] = q * (e0.x * e1.x - e0i * e1i);
      pi[slot] = q * (e0.x * e1i + e0i * e1.x);
    }
    for (int k = cd.w; k < kend; k++) {
      const int g2 = cd.z + (k - cd.w);
      const double pref = D.k[k].w;
      const double2 Sk = S[k];
      double oc = 0.0, os = 0.0, nc = 0.0, ns = 0.0;
#pragma unroll
      for (int slot = 0; slot < 2 * MC_MAXG; slot++) {
        if (slot < sbeg || slot >= send) continue;
        const double2 e2 = sh_tab[slot][2][g2];
        const double c = pr[slot] * e2.x - pi[slot] * e2.y, sn = pr[slot] * e2.y + pi[slot] * e2.x;
        if (slot < M) {
          oc += c;
          os += sn;
        } else {
          nc += c;
          ns += sn;
        }
      }
      if (has_old) ro += ((Sk.x - oc) * oc + (Sk.y - os) * os) * pref;
      if (has_new) {
        const double bc = (kind == MC_TRANSLATE) ? Sk.x - oc : Sk.x;
        const double bs = (kind == MC_TRANSLATE) ? Sk.y - os : Sk.y;
        rn += (bc * nc + bs * ns) * pref;
      }
    }
  }
  } else {
    // mixed: the same sums in double-float arithmetic on per-atom FP32 hi + lo
    // tables (from FP64 sincospi) and the chain's S split per launch
    const int G0 = D.gmax[0], G1 = D.gmax[1], G2 = D.gmax[2];
    const int nt = G0 + G1 + G2 + 3;
    for (int i = threadIdx.x; i < 2 * M * nt; i += MC_TB) {
      const int slot = i / nt;
      int r = i - slot * nt;
      int axis = 0;
      if (r > G0) {
        r -= G0 + 1;
        axis = 1;
        if (r > G1) {
          r -= G1 + 1;
          axis = 2;
        }
      }
      const bool is_new = slot >= M;
      if (is_new ? has_new : has_old) {
        const double f = (is_new ? sh_fnew : sh_fold)[3 * (slot % M) + axis];
        double sn, cs;
        sincospi(2.0 * r * f, &sn, &cs);
        const float ch = (float)cs, sh = (float)sn;
        sh_tabf[slot][axis][r] = make_float4(ch, sh, (float)(cs - (double)ch), (float)(sn - (double)sh));
      }
    }
    __syncthreads();
    McFF fro{0.f, 0.f}, frn{0.f, 0.f};
    const float4 *Sf = D.Sff + (int64_t)chain * D.nk;
    const int sbeg = has_old ? 0 : M, send = has_new ? 2 * M : M;
    for (int col = threadIdx.x; col < D.ncol; col += MC_TB) {
      const int4 cd = D.cols[col];
      const int kend = D.cols[col + 1].w;
      const int a0 = cd.x < 0 ? -cd.x : cd.x, a1 = cd.y < 0 ? -cd.y : cd.y;
      const float s0 = cd.x < 0 ? -1.f : 1.f, s1 = cd.y < 0 ? -1.f : 1.f;
      McFF pr[2 * MC_MAXG], pim[2 * MC_MAXG];
#pragma unroll
      for (int slot = 0; slot < 2 * MC_MAXG; slot++) {
        if (slot < sbeg || slot >= send) continue;
        const float4 t0 = sh_tabf[slot][0][a0], t1 = sh_tabf[slot][1][a1];
        const McFF e0r{t0.x, t0.z}, e0i{s0 * t0.y, s0 * t0.w}, e1r{t1.x, t1.z}, e1i{s1 * t1.y, s1 * t1.w};
        const McFF q{D.gqh[slot % M], D.gql[slot % M]};
        const McFF xr = ff_add(ff_mul(e0r, e1r), ff_neg(ff_mul(e0i, e1i)));
        const McFF xi = ff_add(ff_mul(e0r, e1i), ff_mul(e0i, e1r));
        pr[slot] = ff_mul(q, xr);
        pim[slot] = ff_mul(q, xi);
      }
      for (int k = cd.w; k < kend; k++) {
        const int g2 = cd.z + (k - cd.w);
        const float2 pk = D.kpf[k];
        const McFF pref{pk.x, pk.y};
        const float4 sq = Sf[k];
        const McFF Sr{sq.x, sq.z}, Si{sq.y, sq.w};
        McFF oc{0.f, 0.f}, os{0.f, 0.f}, nc{0.f, 0.f}, ns{0.f, 0.f};
#pragma unroll
        for (int slot = 0; slot < 2 * MC_MAXG; slot++) {
          if (slot < sbeg || slot >= send) continue;
          const float4 t2 = sh_tabf[slot][2][g2];
          const McFF er{t2.x, t2.z}, ei{t2.y, t2.w};
          if (slot < M) {
            ff_acc(oc, pr[slot], er);
            ff_acc(oc, ff_neg(pim[slot]), ei);
            ff_acc(os, pr[slot], ei);
            ff_acc(os, pim[slot], er);
          } else {
            ff_acc(nc, pr[slot], er);
            ff_acc(nc, ff_neg(pim[slot]), ei);
            ff_acc(ns, pr[slot], ei);
            ff_acc(ns, pim[slot], er);
          }
        }
        if (has_old) {
          const McFF t = ff_add(ff_mul(ff_add(Sr, ff_neg(oc)), oc), ff_mul(ff_add(Si, ff_neg(os)), os));
          fro = ff_add(fro, ff_mul(t, pref));
        }
        if (has_new) {
          const McFF bc = (kind == MC_TRANSLATE) ? ff_add(Sr, ff_neg(oc)) : Sr;
          const McFF bs = (kind == MC_TRANSLATE) ? ff_add(Si, ff_neg(os)) : Si;
          const McFF t = ff_add(ff_mul(bc, nc), ff_mul(bs, ns));
          frn = ff_add(frn, ff_mul(t, pref));
        }
      }
    }
    ro = (double)fro.h + (double)fro.l;
    rn = (double)frn.h + (double)frn.l;
  }
  // deterministic block reduction: 4 energies, 2 reciprocal sums (added),
  // 4 smallest distances (min)
  double v[10];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    v[q] = acc[q].value();
    v[6 + q] = F64 ? acc[q].dmin2 : (double)acc[q].dmin2f;
  }
  v[4] = ro;
  v[5] = rn;
#pragma unroll
  for (int q = 0; q < 10; q++)
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) {
      const double y = __shfl_down_sync(0xffffffffu, v[q], o);
      v[q] = (q < 6) ? v[q] + y : fmin(v[q], y);
    }
  if ((threadIdx.x & 31) == 0)
#pragma unroll
    for (int q = 0; q < 10; q++) red[threadIdx.x >> 5][q] = v[q];
  __syncthreads();
  if (threadIdx.x == 0) {
    double s[10];
    for (int q = 0; q < 10; q++) s[q] = red[0][q];
    for (int w = 1; w < MC_TB / 32; w++)
      for (int q = 0; q < 10; q++) s[q] = (q < 6) ? s[q] + red[w][q] : fmin(s[q], red[w][q]);
    const double cc2 = D.close2;
    double e = 0.0;
    if (has_old) {
      const double eh = (s[6] < cc2) ? 1e10 : s[0];
      const double eg = (s[7] < cc2) ? 1e10 : s[1];
      e -= eg + eh + 2.0 * s[4] * D.inv_diel;
    }
    if (has_new) {
      const double eh = (s[8] < cc2) ? 1e10 : s[2];
      const double eg = (s[9] < cc2) ? 1e10 : s[3];
      e += eg + eh + 2.0 * s[5] * D.inv_diel;
    }
    energy[t] = e;
  }
}

// Structure-factor change of accepted trials: S[chain] += dS_new - dS_old,
// FP64 in the reference's op order (its accept() adds the trial's factors).
__global__ void k_mc_apply_sfac(const McDev D, const int4 *__restrict__ trials, const int *__restrict__ which,
                                int napply, const double *__restrict__ newpos, double2 *__restrict__ S) {
  const int k = blockIdx.x * blockDim.x + threadIdx.x;
  const int u = blockIdx.y;
  if (k >= D.nk || u >= napply) return;
  const int t = which[u];
  const int4 tr = trials[t];
  const int M = D.M;
  const double4_32a K = D.k[k];
  double dc = 0.0, ds = 0.0;
  if (tr.y != MC_INSERT) {
    const double *p = D.gpos + (((int64_t)tr.x * D.max_guests + tr.z) * M) * 3;
    double c = 0.0, s = 0.0;
    for (int a = 0; a < M; a++) {
      double cc, ss;
      mc_phase<true>(K, p + 3 * a, D.gq[a], cc, ss);
      c = xadd(c, cc);
      s = xadd(s, ss);
    }
    dc -= c;
    ds -= s;
  }
  if (tr.y != MC_DELETE) {
    const double *p = newpos + (int64_t)t * M * 3;
    double c = 0.0, s = 0.0;
    for (int a = 0; a < M; a++) {
      double cc, ss;
      mc_phase<true>(K, p + 3 * a, D.gq[a], cc, ss);
      c = xadd(c, cc);
      s = xadd(s, ss);
    }
    dc += c;
    ds += s;
  }
  double2 *Sk = S + (int64_t)tr.x * D.nk + k;
  *Sk = make_double2(Sk->x + dc, Sk->y + ds);
}

// Guest positions of accepted trials (after the structure factors, which
// read the old positions): insert appends, delete moves the last guest into
// the freed slot, translate overwrites.  One thread per (applied trial,
// coordinate); dst/src slots are resolved on the host.
__global__ void k_mc_apply_pos(const int4 *__restrict__ moves, int nmove, const double *__restrict__ newpos, int M,
                               double *__restrict__ gpos, int64_t max_guests) {
  const int u = blockIdx.x;
  const int i = threadIdx.x;
  if (u >= nmove || i >= 3 * M) return;
  const int4 mv = moves[u];  // chain, dst slot, src slot (-1: from newpos[trial]), trial
  const int64_t dst = (((int64_t)mv.x * max_guests + mv.y) * M) * 3 + i;
  if (mv.z < 0)
    gpos[dst] = newpos[(int64_t)mv.w * M * 3 + i];
  else
    gpos[dst] = gpos[(((int64_t)mv.x * max_guests + mv.z) * M) * 3 + i];
}

// 2 sum pref (cos dcos + sin dsin) (ewald.c:508-522): strided per-thread
// sums, combined in a fixed order.
__global__ void k_mc_deltae(const double *__restrict__ pref, const double *__restrict__ dc, const double *__restrict__ c,
                            const double *__restrict__ ds, const double *__restrict__ s, int64_t nk,
                            double *__restrict__ out) {
  __shared__ double red[256];
  double e = 0.0;
  for (int64_t i = threadIdx.x; i < nk; i += blockDim.x) e += (c[i] * dc[i] + s[i] * ds[i]) * pref[i];
  red[threadIdx.x] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double t = 0.0;
    for (int i = 0; i < (int)blockDim.x; i++) t += red[i];
    *out = 2.0 * t;
  }
}

McDev make_dev(const yg_mc *mc) {
  McDev D;
  D.cell = mc->cell;
  for (int a = 0; a < 3; a++) D.rmax[a] = mc->rmax[a];
  for (int a = 0; a < 9; a++) D.rvf[a] = (float)mc->cell.rv[a];
  D.rc2 = mc->rcut * mc->rcut;
  D.rc2f = (float)D.rc2;
  D.alpha = mc->alpha;
  D.inv_diel = 1.0 / mc->diel;
  D.alphaf = (float)mc->alpha;
  D.inv_dielf = (float)(1.0 / mc->diel);
  D.close2 = mc->close_contact >= 0.0 ? mc->close_contact * mc->close_contact : -1.0;
  const double dnear = 2.0 / mc->alpha;  // erfc(alpha d) = 4.7e-3 there
  D.near2f = (float)(dnear * dnear);
  D.rc2f_lo = (float)(D.rc2 * (1.0 - 1e-6));
  D.rc2f_hi = (float)(D.rc2 * (1.0 + 1e-6));
  for (int a = 0; a < 3; a++) D.gmax[a] = (int)mc->gmax[a];
  D.kg = mc->d_kg;
  D.nk = mc->nk;
  D.k = mc->d_k;
  D.nframe = mc->nframe;
  D.fpos = mc->d_fpos;
  D.ffrac = mc->d_ffrac;
  D.ffix = mc->d_ffix;
  D.gfix = mc->d_gfix;
  D.cols = mc->d_cols;
  D.ncol = mc->ncol;
  D.fpar = mc->d_fpar;
  D.M = mc->M;
  for (int a = 0; a < MC_MAXG; a++) {
    D.gq[a] = a < mc->M ? mc->gq[a] : 0.0;
    D.gsig[a] = a < mc->M ? mc->gsig[a] : 0.0;
    D.gseps[a] = a < mc->M ? mc->gseps[a] : 0.0;
    D.gpar[a][0] = D.gq[a];
    D.gpar[a][1] = D.gsig[a];
    D.gpar[a][2] = D.gseps[a];
    D.gqf[a] = (float)D.gq[a];
    D.gsigf[a] = (float)D.gsig[a];
    D.gsepsf[a] = (float)D.gseps[a];
  }
  D.fparf = mc->d_fparf;
  D.max_guests = mc->max_guests;
  D.gpos = mc->d_gpos;
  D.gfrac = mc->d_gfrac;
  D.nguest = mc->d_nguest;
  D.S = mc->d_S;
  D.Sff = mc->d_Sff;
  D.kpf = mc->d_kpf;
  for (int a = 0; a < MC_MAXG; a++) {
    const double q = a < mc->M ? mc->gq[a] : 0.0;
    D.gqh[a] = (float)q;
    D.gql[a] = (float)(q - (double)D.gqh[a]);
  }
  return D;
}

int mc_alloc(void **p, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMalloc(p, bytes);
  if (e != cudaSuccess) {
    *p = nullptr;
    return yg_cuda_fail(e, "cudaMalloc");
  }
  return YG_OK;
}

// The k vectors of the half sphere in the reference's loop order, with
// their prefactors (ewald.c:441-471, same operation order) and their
// element in the dense layout.
void mc_kvectors(const double *gv, double volume, double alpha, const int64_t *gmax, double gcut,
                 std::vector<double4_32a> &kv, std::vector<int64_t> &kidx, std::vector<double> *dense,
                 std::vector<int4> *kg = nullptr) {
  const double two_pi = 6.283185307179586476925;
  const double four_pi = 12.56637061435917295385;
  double kvecs[9];
  for (int i = 0; i < 9; i++) kvecs[i] = two_pi * gv[i];
  const double fac1 = four_pi / volume;
  const double fac2 = 0.25 / alpha / alpha;
  double gc = gcut * two_pi;
  gc *= gc;
  int64_t index = 0;
  if (dense) dense->assign((size_t)((2 * gmax[0] + 1) * (2 * gmax[1] + 1) * (gmax[2] + 1)), 0.0);
  for (int64_t g0 = -gmax[0]; g0 <= gmax[0]; g0++)
    for (int64_t g1 = -gmax[1]; g1 <= gmax[1]; g1++)
      for (int64_t g2 = 0; g2 <= gmax[2]; g2++) {
        index++;
        if (g2 == 0) {
          if (g1 < 0) continue;
          if (g1 == 0 && g0 <= 0) continue;
        }
        double k[3];
        k[0] = (g0 * kvecs[0] + g1 * kvecs[3] + g2 * kvecs[6]);
        k[1] = (g0 * kvecs[1] + g1 * kvecs[4] + g2 * kvecs[7]);
        k[2] = (g0 * kvecs[2] + g1 * kvecs[5] + g2 * kvecs[8]);
        const double ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
        if (ksq > gc) continue;
        const double p = fac1 * exp(-ksq * fac2) / ksq;
        kv.push_back(make_double4_32a(k[0], k[1], k[2], p));
        kidx.push_back(index);
        if (kg) kg->push_back(make_int4((int)g0, (int)g1, (int)g2, 0));
        // the reference's store lands one past the array for the last loop
        // index; that element does not exist here
        if (dense && index < (int64_t)dense->size()) (*dense)[index] = p;
      }
}

// Structure factors of natom atoms (charges q, or the guest template) into
// out[k] (+ base[k] when base is given), on the context's stream.
int mc_sfac(yg_mc *mc, const double *d_pos, const double *d_q, int64_t natom, const double2 *base, double2 *out) {
  const int nk = mc->nk;
  const int nchunk = (int)std::max<int64_t>(1, (natom + MC_SF_CHUNK - 1) / MC_SF_CHUNK);
  size_t need = (size_t)nchunk * nk * sizeof(double2);
  if (need > mc->spart_cap) {
    if (mc->d_Spart) cudaFree(mc->d_Spart);
    int rc = mc_alloc((void **)&mc->d_Spart, need);
    if (rc) return rc;
    mc->spart_cap = need;
  }
  McDev D = make_dev(mc);
  if (natom > 0) {
    dim3 grid((nk + 127) / 128, nchunk);
    k_mc_sfac_part<<<grid, 128, 0, mc->stream>>>(mc->d_k, nk, d_pos, d_q, D, natom, mc->d_Spart);
    mc->launches++;
    k_mc_sfac_sum<<<(nk + 127) / 128, 128, 0, mc->stream>>>(mc->d_Spart, nchunk, nk, base, out);
  } else {
    k_mc_sfac_sum<<<(nk + 127) / 128, 128, 0, mc->stream>>>(mc->d_Spart, 0, nk, base, out);
  }
  mc->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return yg_cuda_fail(e, "k_mc_sfac");
  return YG_OK;
}

int mc_check_cell(const double *rvecs, const double *gvecs, double volume) {
  if (!rvecs || !gvecs || !(volume > 0.0)) {
    yg_set_error("a 3D periodic cell is required");
    return YG_ERR_ARG;
  }
  return YG_OK;
}

}  // namespace

extern "C" {

int yg_ewald_prefactors(const double *gvecs, double volume, double alpha, const int64_t *gmax, double gcut,
                        double *prefactors) {
  if (!gvecs || !gmax || !prefactors || !(alpha > 0.0) || !(volume > 0.0)) return YG_ERR_ARG;
  for (int a = 0; a < 3; a++)
    if (gmax[a] < 0 || gmax[a] > 4096) return YG_ERR_ARG;
  std::vector<double4_32a> kv;
  std::vector<int64_t> kidx;
  std::vector<double> dense;
  mc_kvectors(gvecs, volume, alpha, gmax, gcut, kv, kidx, &dense);
  memcpy(prefactors, dense.data(), dense.size() * sizeof(double));
  return YG_OK;
}

int yg_ewald_structurefactors(const double *pos, int64_t natom, const double *charges, const double *rvecs,
                              const double *gvecs, double volume, const int64_t *gmax, double gcut,
                              double *cosfacs, double *sinfacs, void *stream) {
  if ((natom > 0 && (!pos || !charges)) || natom < 0 || !gmax || !cosfacs || !sinfacs) return YG_ERR_ARG;
  int rc = mc_check_cell(rvecs, gvecs, volume);
  if (rc) return rc;
  yg_mc tmp;
  tmp.stream = (cudaStream_t)stream;
  memcpy(tmp.cell.rv, rvecs, 9 * sizeof(double));
  memcpy(tmp.cell.gv, gvecs, 9 * sizeof(double));
  tmp.cell.volume = volume;
  tmp.cell.nvec = 3;
  std::vector<double4_32a> kv;
  mc_kvectors(gvecs, volume, 1.0, gmax, gcut, kv, tmp.kidx, nullptr);
  tmp.nk = (int)kv.size();
  tmp.M = 1;
  double *d_pos = nullptr, *d_q = nullptr;
  double2 *d_out = nullptr;
  std::vector<double2> h(tmp.nk > 0 ? tmp.nk : 1);
  rc = mc_alloc((void **)&tmp.d_k, kv.size() * sizeof(double4_32a) + 16);
  if (!rc) rc = mc_alloc((void **)&d_pos, (size_t)natom * 3 * sizeof(double));
  if (!rc) rc = mc_alloc((void **)&d_q, (size_t)natom * sizeof(double));
  if (!rc) rc = mc_alloc((void **)&d_out, h.size() * sizeof(double2));
  if (!rc && tmp.nk > 0) {
    cudaError_t e = cudaMemcpyAsync(tmp.d_k, kv.data(), kv.size() * sizeof(double4_32a), cudaMemcpyHostToDevice, tmp.stream);
    if (e == cudaSuccess && natom > 0)
      e = cudaMemcpyAsync(d_pos, pos, (size_t)natom * 3 * sizeof(double), cudaMemcpyHostToDevice, tmp.stream);
    if (e == cudaSuccess && natom > 0)
      e = cudaMemcpyAsync(d_q, charges, (size_t)natom * sizeof(double), cudaMemcpyHostToDevice, tmp.stream);
    if (e != cudaSuccess) rc = yg_cuda_fail(e, "cudaMemcpyAsync");
    if (!rc) rc = mc_sfac(&tmp, d_pos, d_q, natom, nullptr, d_out);
    if (!rc) {
      e = cudaMemcpyAsync(h.data(), d_out, tmp.nk * sizeof(double2), cudaMemcpyDeviceToHost, tmp.stream);
      if (e == cudaSuccess) e = cudaStreamSynchronize(tmp.stream);
      if (e != cudaSuccess) rc = yg_cuda_fail(e, "readback");
    }
  }
  if (!rc) {
    const int64_t ndense = (2 * gmax[0] + 1) * (2 * gmax[1] + 1) * (gmax[2] + 1);
    for (int k = 0; k < tmp.nk; k++) {
      const int64_t i = tmp.kidx[k];
      if (i >= ndense) continue;
      cosfacs[i] += h[k].x;
      sinfacs[i] += h[k].y;
    }
  }
  cudaFree(tmp.d_k);
  tmp.d_k = nullptr;
  cudaFree(tmp.d_Spart);
  tmp.d_Spart = nullptr;
  cudaFree(d_pos);
  cudaFree(d_q);
  cudaFree(d_out);
  return rc;
}

int yg_ewald_deltae(const double *prefactors, const double *deltacosfacs, const double *cosfacs,
                    const double *deltasinfacs, const double *sinfacs, int64_t nk, double *out) {
  if (!prefactors || !deltacosfacs || !cosfacs || !deltasinfacs || !sinfacs || !out || nk < 0) return YG_ERR_ARG;
  double *d = nullptr;
  const size_t n = (size_t)std::max<int64_t>(nk, 1);
  int rc = mc_alloc((void **)&d, (5 * n + 1) * sizeof(double));
  if (rc) return rc;
  const double *src[5] = {prefactors, deltacosfacs, cosfacs, deltasinfacs, sinfacs};
  cudaError_t e = cudaSuccess;
  for (int i = 0; i < 5 && e == cudaSuccess && nk > 0; i++)
    e = cudaMemcpy(d + i * n, src[i], nk * sizeof(double), cudaMemcpyHostToDevice);
  if (e == cudaSuccess) {
    k_mc_deltae<<<1, 256>>>(d, d + n, d + 2 * n, d + 3 * n, d + 4 * n, nk, d + 5 * n);
    e = cudaGetLastError();
  }
  if (e == cudaSuccess) e = cudaMemcpy(out, d + 5 * n, sizeof(double), cudaMemcpyDeviceToHost);
  cudaFree(d);
  if (e != cudaSuccess) return yg_cuda_fail(e, "yg_ewald_deltae");
  return YG_OK;
}

int yg_mc_create(const double *rvecs, const double *gvecs, double volume, const int64_t *rmax, double rcut,
                 double alpha, double gcut, const int64_t *gmax, double dielectric, double close_contact,
                 int64_t nframe,
                 const double *frame_pos, const double *frame_charges, const double *frame_sigma,
                 const double *frame_epsilon, int64_t guest_natom, const double *guest_charges,
                 const double *guest_sigma, const double *guest_epsilon, int64_t nchain, int64_t max_guests,
                 int precision, void *stream, yg_mc **out) {
  if (!out || !rmax || !gmax || nframe < 0 || guest_natom < 1 || guest_natom > MC_MAXG || nchain < 1 ||
      max_guests < 1 || !(rcut > 0.0) || !(alpha > 0.0) || !(dielectric > 0.0) || !guest_charges ||
      !guest_sigma || !guest_epsilon || (nframe > 0 && (!frame_pos || !frame_charges || !frame_sigma ||
                                                         !frame_epsilon)))
    return YG_ERR_ARG;
  if (precision != YG_FP64 && precision != YG_MIXED) {
    yg_set_error("MC trials support the fp64 and mixed modes");
    return YG_ERR_ARG;
  }
  int rc = mc_check_cell(rvecs, gvecs, volume);
  if (rc) return rc;
  for (int a = 0; a < 3; a++)
    if (rmax[a] < 0 || rmax[a] > 8 || gmax[a] < 0 || gmax[a] > 1024) return YG_ERR_ARG;
  for (int a = 0; a < 3; a++)
    if (gmax[a] >= MC_GT) {
      yg_set_error("MC trials support gmax <= 23 per axis");
      return YG_ERR_UNSUPPORTED;
    }
  yg_mc *mc = new yg_mc();
  mc->precision = precision;
  mc->stream = (cudaStream_t)stream;
  memcpy(mc->cell.rv, rvecs, 9 * sizeof(double));
  memcpy(mc->cell.gv, gvecs, 9 * sizeof(double));
  mc->cell.volume = volume;
  mc->cell.nvec = 3;
  for (int a = 0; a < 3; a++) {
    mc->rmax[a] = (int)rmax[a];
    mc->gmax[a] = gmax[a];
  }
  mc->rcut = rcut;
  mc->alpha = alpha;
  mc->gcut = gcut;
  mc->diel = dielectric;
  mc->close_contact = close_contact;
  mc->nframe = nframe;
  mc->M = (int)guest_natom;
  for (int a = 0; a < mc->M; a++) {
    if (guest_epsilon[a] < 0.0) {
      delete mc;
      return YG_ERR_ARG;
    }
    mc->gq[a] = guest_charges[a];
    mc->gsig[a] = guest_sigma[a];
    mc->gseps[a] = std::sqrt(guest_epsilon[a]);
  }
  mc->nchain = nchain;
  mc->max_guests = max_guests;
  mc->nguest.assign(nchain, 0);
  std::vector<double4_32a> kv;
  std::vector<int4> kg;
  mc_kvectors(gvecs, volume, alpha, gmax, gcut, kv, mc->kidx, &mc->pref_dense, &kg);
  mc->nk = (int)kv.size();
  // columns: runs of consecutive k with the same (g0, g1); their g2 values
  // are consecutive (|k|^2 is convex in g2)
  std::vector<int4> cols;
  for (int k = 0; k < mc->nk; k++)
    if (k == 0 || kg[k].x != kg[k - 1].x || kg[k].y != kg[k - 1].y) cols.push_back(make_int4(kg[k].x, kg[k].y, kg[k].z, k));
  mc->ncol = (int)cols.size();
  cols.push_back(make_int4(0, 0, 0, mc->nk));
  const size_t NG = (size_t)nchain * max_guests * mc->M;
  std::vector<double4_32a> fpar(nframe > 0 ? nframe : 1);
  for (int64_t i = 0; i < nframe; i++) {
    if (frame_epsilon[i] < 0.0) {
      delete mc;
      return YG_ERR_ARG;
    }
    fpar[i] = make_double4_32a(frame_charges[i], frame_sigma[i], std::sqrt(frame_epsilon[i]), 0.0);
  }
  rc = mc_alloc((void **)&mc->d_k, kv.size() * sizeof(double4_32a) + 16);
  if (!rc) rc = mc_alloc((void **)&mc->d_kg, kg.size() * sizeof(int4) + 16);
  if (!rc) rc = mc_alloc((void **)&mc->d_fpos, (size_t)nframe * 3 * sizeof(double));
  if (!rc) rc = mc_alloc((void **)&mc->d_ffrac, (size_t)nframe * 3 * sizeof(double));
  if (!rc) rc = mc_alloc((void **)&mc->d_ffix, (size_t)nframe * 3 * sizeof(unsigned));
  if (!rc) rc = mc_alloc((void **)&mc->d_gfix, NG * 3 * sizeof(unsigned));
  if (!rc) rc = mc_alloc((void **)&mc->d_cols, cols.size() * sizeof(int4));
  if (!rc) rc = mc_alloc((void **)&mc->d_fpar, fpar.size() * sizeof(double4_32a));
  std::vector<float4> fparf(fpar.size());
  for (size_t i = 0; i < fpar.size(); i++)
    fparf[i] = make_float4((float)fpar[i].x, (float)fpar[i].y, (float)fpar[i].z, 0.0f);
  if (!rc) rc = mc_alloc((void **)&mc->d_fparf, fparf.size() * sizeof(float4));
  if (!rc) rc = mc_alloc((void **)&mc->d_gpos, NG * 3 * sizeof(double));
  if (!rc) rc = mc_alloc((void **)&mc->d_gfrac, NG * 3 * sizeof(double));
  if (!rc) rc = mc_alloc((void **)&mc->d_nguest, (size_t)nchain * sizeof(int));
  if (!rc) rc = mc_alloc((void **)&mc->d_S, (size_t)nchain * std::max(1, mc->nk) * sizeof(double2));
  if (!rc) rc = mc_alloc((void **)&mc->d_Sff, (size_t)nchain * std::max(1, mc->nk) * sizeof(float4));
  if (!rc) rc = mc_alloc((void **)&mc->d_kpf, (size_t)std::max(1, mc->nk) * sizeof(float2));
  std::vector<float2> kpf(std::max(1, mc->nk));
  for (int k = 0; k < mc->nk; k++) {
    const float h = (float)kv[k].w;
    kpf[k] = make_float2(h, (float)(kv[k].w - (double)h));
  }
  if (!rc) rc = mc_alloc((void **)&mc->d_Sframe, (size_t)std::max(1, mc->nk) * sizeof(double2));
  cudaError_t e = cudaSuccess;
  if (!rc) {
    if (mc->nk > 0) e = cudaMemcpyAsync(mc->d_k, kv.data(), kv.size() * sizeof(double4_32a), cudaMemcpyHostToDevice, mc->stream);
    if (e == cudaSuccess && mc->nk > 0)
      e = cudaMemcpyAsync(mc->d_kpf, kpf.data(), mc->nk * sizeof(float2), cudaMemcpyHostToDevice, mc->stream);
    if (e == cudaSuccess && mc->nk > 0)
      e = cudaMemcpyAsync(mc->d_kg, kg.data(), kg.size() * sizeof(int4), cudaMemcpyHostToDevice, mc->stream);
    if (e == cudaSuccess && nframe > 0)
      e = cudaMemcpyAsync(mc->d_fpos, frame_pos, (size_t)nframe * 3 * sizeof(double), cudaMemcpyHostToDevice, mc->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(mc->d_fpar, fpar.data(), fpar.size() * sizeof(double4_32a), cudaMemcpyHostToDevice, mc->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(mc->d_fparf, fparf.data(), fparf.size() * sizeof(float4), cudaMemcpyHostToDevice, mc->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(mc->d_nguest, 0, (size_t)nchain * sizeof(int), mc->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(mc->d_gpos, 0, NG * 3 * sizeof(double), mc->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(mc->d_gfrac, 0, NG * 3 * sizeof(double), mc->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(mc->d_gfix, 0, NG * 3 * sizeof(unsigned), mc->stream);
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(mc->d_cols, cols.data(), cols.size() * sizeof(int4), cudaMemcpyHostToDevice, mc->stream);
    if (e != cudaSuccess) rc = yg_cuda_fail(e, "yg_mc_create upload");
  }
  if (!rc && nframe > 0) {
    k_mc_frac<<<yg_blocks(nframe, 256), 256, 0, mc->stream>>>(mc->d_fpos, nframe, mc->cell, mc->d_ffrac, mc->d_ffix);
    mc->launches++;
  }
  if (!rc && mc->nk > 0) rc = mc_sfac(mc, mc->d_fpos, nullptr, 0, nullptr, mc->d_Sframe);
  if (!rc && mc->nk > 0 && nframe > 0) {
    // framework charges per atom
    double *d_q = nullptr;
    std::vector<double> q(frame_charges, frame_charges + nframe);
    rc = mc_alloc((void **)&d_q, nframe * sizeof(double));
    if (!rc) {
      e = cudaMemcpyAsync(d_q, q.data(), nframe * sizeof(double), cudaMemcpyHostToDevice, mc->stream);
      if (e != cudaSuccess) rc = yg_cuda_fail(e, "cudaMemcpyAsync");
    }
    if (!rc) rc = mc_sfac(mc, mc->d_fpos, d_q, nframe, nullptr, mc->d_Sframe);
    if (!rc) {
      e = cudaStreamSynchronize(mc->stream);
      if (e != cudaSuccess) rc = yg_cuda_fail(e, "cudaStreamSynchronize");
    }
    cudaFree(d_q);
  }
  // every chain starts empty: S = S_frame
  for (int64_t c = 0; !rc && c < nchain && mc->nk > 0; c++) {
    e = cudaMemcpyAsync(mc->d_S + c * mc->nk, mc->d_Sframe, mc->nk * sizeof(double2), cudaMemcpyDeviceToDevice,
                        mc->stream);
    if (e != cudaSuccess) rc = yg_cuda_fail(e, "cudaMemcpyAsync");
  }
  if (!rc) {
    e = cudaStreamSynchronize(mc->stream);
    if (e != cudaSuccess) rc = yg_cuda_fail(e, "cudaStreamSynchronize");
  }
  if (rc) {
    yg_mc_destroy(mc);
    return rc;
  }
  *out = mc;
  return YG_OK;
}

int yg_mc_destroy(yg_mc *mc) {
  if (!mc) return YG_OK;
  cudaStreamSynchronize(mc->stream);
  void *bufs[] = {mc->d_fparf,  mc->d_ffix,   mc->d_gfix,   mc->d_cols,   mc->d_kg,     mc->d_k,      mc->d_fpos,   mc->d_ffrac,  mc->d_fpar,     mc->d_gpos,   mc->d_gfrac,
                  mc->d_nguest, mc->d_S,      mc->d_Sframe, mc->d_Spart,    mc->d_trials, mc->d_newpos,
                  mc->d_energy, mc->d_Sff,    mc->d_kpf};
  for (void *b : bufs)
    if (b) cudaFree(b);
  delete mc;
  return YG_OK;
}

int yg_mc_set_precision(yg_mc *mc, int precision) {
  if (!mc || (precision != YG_FP64 && precision != YG_MIXED)) return YG_ERR_ARG;
  mc->precision = precision;
  return YG_OK;
}

int yg_mc_set_chain(yg_mc *mc, int64_t chain, int64_t nguest, const double *guest_pos) {
  if (!mc || chain < 0 || chain >= mc->nchain || nguest < 0 || nguest > mc->max_guests ||
      (nguest > 0 && !guest_pos))
    return YG_ERR_ARG;
  const int64_t off = chain * mc->max_guests * mc->M;
  const int64_t na = nguest * mc->M;
  if (na > 0) {
    YG_CUDA(cudaMemcpyAsync(mc->d_gpos + off * 3, guest_pos, (size_t)na * 3 * sizeof(double), cudaMemcpyHostToDevice,
                            mc->stream));
    k_mc_frac<<<yg_blocks(na, 256), 256, 0, mc->stream>>>(mc->d_gpos + off * 3, na, mc->cell, mc->d_gfrac + off * 3,
                                                           mc->d_gfix + off * 3);
    mc->launches++;
  }
  int ng = (int)nguest;
  YG_CUDA(cudaMemcpyAsync(mc->d_nguest + chain, &ng, sizeof(int), cudaMemcpyHostToDevice, mc->stream));
  int rc;
  if (mc->nk > 0 && (rc = mc_sfac(mc, mc->d_gpos + off * 3, nullptr, na, mc->d_Sframe, mc->d_S + chain * mc->nk)))
    return rc;
  YG_CUDA(cudaStreamSynchronize(mc->stream));
  mc->nguest[chain] = ng;
  return YG_OK;
}

int yg_mc_get_chain(yg_mc *mc, int64_t chain, int64_t *nguest, double *guest_pos, double *cosfacs,
                    double *sinfacs) {
  if (!mc || chain < 0 || chain >= mc->nchain) return YG_ERR_ARG;
  const int64_t ng = mc->nguest[chain];
  if (nguest) *nguest = ng;
  if (guest_pos && ng > 0)
    YG_CUDA(cudaMemcpyAsync(guest_pos, mc->d_gpos + chain * mc->max_guests * mc->M * 3,
                            (size_t)ng * mc->M * 3 * sizeof(double), cudaMemcpyDeviceToHost, mc->stream));
  std::vector<double2> h(mc->nk > 0 ? mc->nk : 1);
  if ((cosfacs || sinfacs) && mc->nk > 0)
    YG_CUDA(cudaMemcpyAsync(h.data(), mc->d_S + chain * mc->nk, mc->nk * sizeof(double2), cudaMemcpyDeviceToHost,
                            mc->stream));
  YG_CUDA(cudaStreamSynchronize(mc->stream));
  if (cosfacs || sinfacs) {
    const size_t nd = mc->pref_dense.size();
    if (cosfacs) memset(cosfacs, 0, nd * sizeof(double));
    if (sinfacs) memset(sinfacs, 0, nd * sizeof(double));
    for (int k = 0; k < mc->nk; k++) {
      const int64_t i = mc->kidx[k];
      if (i >= (int64_t)nd) continue;
      if (cosfacs) cosfacs[i] = h[k].x;
      if (sinfacs) sinfacs[i] = h[k].y;
    }
  }
  return YG_OK;
}

int yg_mc_prefactors(yg_mc *mc, double *prefactors, int64_t *nk_dense) {
  if (!mc) return YG_ERR_ARG;
  if (nk_dense) *nk_dense = (int64_t)mc->pref_dense.size();
  if (prefactors) memcpy(prefactors, mc->pref_dense.data(), mc->pref_dense.size() * sizeof(double));
  return YG_OK;
}

int yg_mc_trials(yg_mc *mc, int64_t ntrial, const int32_t *chain, const int32_t *kind, const int32_t *guest,
                 const double *newpos, double *energy) {
  if (!mc || ntrial < 0 || (ntrial > 0 && (!chain || !kind || !guest || !energy))) return YG_ERR_ARG;
  if (ntrial > (1 << 24)) return YG_ERR_CAPACITY;
  const int M = mc->M;
  mc->h_trials.resize(ntrial);
  mc->h_newpos.assign((size_t)ntrial * M * 3, 0.0);
  for (int64_t t = 0; t < ntrial; t++) {
    const int c = chain[t], k = kind[t], g = guest[t];
    if (c < 0 || c >= mc->nchain || k < MC_INSERT || k > MC_TRANSLATE) {
      yg_set_error("trial with an unknown chain or kind");
      return YG_ERR_ARG;
    }
    if (k != MC_INSERT && (g < 0 || g >= mc->nguest[c])) {
      yg_set_error("deletion or translation of a guest the chain does not hold");
      return YG_ERR_ARG;
    }
    if (k != MC_DELETE) {
      if (!newpos) return YG_ERR_ARG;
      memcpy(&mc->h_newpos[(size_t)t * M * 3], newpos + (size_t)t * M * 3, (size_t)M * 3 * sizeof(double));
    }
    mc->h_trials[t] = make_int4(c, k, k == MC_INSERT ? -1 : g, 0);
  }
  mc->ntrial = ntrial;
  if (ntrial == 0) return YG_OK;
  if (ntrial > mc->cap_trials) {
    if (mc->d_trials) cudaFree(mc->d_trials);
    if (mc->d_newpos) cudaFree(mc->d_newpos);
    if (mc->d_energy) cudaFree(mc->d_energy);
    mc->d_trials = nullptr;
    mc->d_newpos = nullptr;
    mc->d_energy = nullptr;
    mc->cap_trials = 0;
    int64_t cap = ntrial + ntrial / 4 + 64;
    int rc;
    if ((rc = mc_alloc((void **)&mc->d_trials, cap * sizeof(int4)))) return rc;
    if ((rc = mc_alloc((void **)&mc->d_newpos, cap * M * 3 * sizeof(double)))) return rc;
    if ((rc = mc_alloc((void **)&mc->d_energy, cap * sizeof(double)))) return rc;
    mc->cap_trials = cap;
  }
  YG_CUDA(cudaMemcpyAsync(mc->d_trials, mc->h_trials.data(), ntrial * sizeof(int4), cudaMemcpyHostToDevice,
                          mc->stream));
  YG_CUDA(cudaMemcpyAsync(mc->d_newpos, mc->h_newpos.data(), (size_t)ntrial * M * 3 * sizeof(double),
                          cudaMemcpyHostToDevice, mc->stream));
  McDev D = make_dev(mc);
  if (mc->precision == YG_FP64)
    k_mc_trials<true><<<(unsigned)ntrial, MC_TB, 0, mc->stream>>>(D, mc->d_trials, mc->d_newpos, mc->d_energy);
  else {
    if (mc->nk > 0) {
      const int64_t ns = mc->nchain * (int64_t)mc->nk;
      k_mc_split_s<<<(unsigned)((ns + 255) / 256), 256, 0, mc->stream>>>(mc->d_S, ns, mc->d_Sff);
    }
    k_mc_trials<false><<<(unsigned)ntrial, MC_TB, 0, mc->stream>>>(D, mc->d_trials, mc->d_newpos, mc->d_energy);
  }
  mc->launches++;
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return yg_cuda_fail(e, "k_mc_trials");
  YG_CUDA(cudaMemcpyAsync(energy, mc->d_energy, ntrial * sizeof(double), cudaMemcpyDeviceToHost, mc->stream));
  YG_CUDA(cudaStreamSynchronize(mc->stream));
  return YG_OK;
}

int yg_mc_apply(yg_mc *mc, int64_t napply, const int32_t *trial_index) {
  if (!mc || napply < 0 || (napply > 0 && !trial_index)) return YG_ERR_ARG;
  if (napply == 0) return YG_OK;
  const int M = mc->M;
  std::vector<int> which(napply);
  std::vector<char> seen(mc->nchain, 0);
  std::vector<int4> moves;
  std::vector<int> ng = mc->nguest;
  for (int64_t u = 0; u < napply; u++) {
    const int t = trial_index[u];
    if (t < 0 || t >= mc->ntrial) return YG_ERR_ARG;
    const int4 tr = mc->h_trials[t];
    if (seen[tr.x]) {
      yg_set_error("at most one accepted trial per chain and batch");
      return YG_ERR_ARG;
    }
    seen[tr.x] = 1;
    which[u] = t;
    if (tr.y == MC_INSERT) {
      if (ng[tr.x] >= mc->max_guests) {
        yg_set_error("chain is full");
        return YG_ERR_CAPACITY;
      }
      moves.push_back(make_int4(tr.x, ng[tr.x], -1, t));
      ng[tr.x]++;
    } else if (tr.y == MC_TRANSLATE) {
      moves.push_back(make_int4(tr.x, tr.z, -1, t));
    } else {
      const int last = ng[tr.x] - 1;
      if (tr.z != last) moves.push_back(make_int4(tr.x, tr.z, last, t));
      ng[tr.x]--;
    }
  }
  int *d_which = nullptr;
  int4 *d_moves = nullptr;
  int rc = mc_alloc((void **)&d_which, napply * sizeof(int));
  if (!rc) rc = mc_alloc((void **)&d_moves, std::max<size_t>(1, moves.size()) * sizeof(int4));
  if (!rc) {
    cudaError_t e = cudaMemcpyAsync(d_which, which.data(), napply * sizeof(int), cudaMemcpyHostToDevice, mc->stream);
    if (e == cudaSuccess && !moves.empty())
      e = cudaMemcpyAsync(d_moves, moves.data(), moves.size() * sizeof(int4), cudaMemcpyHostToDevice, mc->stream);
    if (e != cudaSuccess) rc = yg_cuda_fail(e, "cudaMemcpyAsync");
  }
  if (!rc) {
    McDev D = make_dev(mc);
    if (mc->nk > 0) {
      dim3 grid((mc->nk + 127) / 128, (unsigned)napply);
      k_mc_apply_sfac<<<grid, 128, 0, mc->stream>>>(D, mc->d_trials, d_which, (int)napply, mc->d_newpos, mc->d_S);
      mc->launches++;
    }
    if (!moves.empty()) {
      k_mc_apply_pos<<<(unsigned)moves.size(), 32, 0, mc->stream>>>(d_moves, (int)moves.size(), mc->d_newpos, M,
                                                                    mc->d_gpos, mc->max_guests);
      mc->launches++;
    }
    // fractional coordinates of every guest slot (cheap; keeps them exact)
    const int64_t NG = mc->nchain * mc->max_guests * M;
    k_mc_frac<<<yg_blocks(NG, 256), 256, 0, mc->stream>>>(mc->d_gpos, NG, mc->cell, mc->d_gfrac, mc->d_gfix);
    mc->launches++;
    std::vector<int> ngi(ng.begin(), ng.end());
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess)
      e = cudaMemcpyAsync(mc->d_nguest, ngi.data(), mc->nchain * sizeof(int), cudaMemcpyHostToDevice, mc->stream);
    if (e == cudaSuccess) e = cudaStreamSynchronize(mc->stream);
    if (e != cudaSuccess) rc = yg_cuda_fail(e, "yg_mc_apply");
    if (!rc) mc->nguest = ng;
  }
  cudaFree(d_which);
  cudaFree(d_moves);
  return rc;
}

int64_t yg_mc_launch_count(yg_mc *mc) { return mc ? mc->launches : -1; }

}  // extern "C"
