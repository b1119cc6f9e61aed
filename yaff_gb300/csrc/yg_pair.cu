// yg_pair.cu -- kernel (b): fused real-space pair potentials.
//
// One traversal of the full neighbour list evaluates every registered pair
// potential (LJ, MM3 exp-6, EI/erfc; yaff/pes/pair_pot.c:277-352, :711-751)
// with exclusion scaling and truncation (pair_pot.c:84-176,
// truncation.c:30-76).  One warp owns one atom: lanes stride over its list
// entries, accumulate the energy, the gradient of the owning atom and the
// virial, and the warp reduces them.  Because the list holds every pair from
// both atoms, each atom's gradient is complete after its own warp finishes:
// no atomics, a deterministic summation order, and each entry contributes
// half the pair energy and virial.
//
// Precision modes: YG_FP64 computes and accumulates in FP64; YG_MIXED
// evaluates the terms in FP32 on cell-local FP32 coordinates (relative
// vectors never exceed a few cutoffs, so FP32 keeps ~1e-7 relative accuracy)
// with per-lane FP32 partial sums that are reduced in FP64 across the warp,
// the block and the grid; YG_MIXED_KAHAN keeps Kahan-compensated FP32 sums.
#include <cmath>
#include <type_traits>

#include "yg_internal.cuh"
#include "yg_pairterm.cuh"

#ifndef YG_PAIR_ATOMS
#define YG_PAIR_ATOMS 4  // atoms per warp at most (energy and virial reduced once per warp)
#endif

namespace {

struct PairArgs {
  int64_t natom;
  int64_t cap;
  const uint2 *nbr;
  const int2 *ncount;         // (front, back) entries of every row
  // the back segment (the skin shell beyond every pair cutoff at the build)
  // is read unless the coordinates are those of the build: fresh is a device
  // flag (nonzero: rebuilt this step) or null, then `back` decides
  const int *fresh;
  int back;
  const int *sorted;
  const double4_32a *x64;
  const float4 *x32;
  const double *shift64;
  const float4 *shift32;
  const double *pp64;
  const float *pp32;
  PairPotDev pot[YG_MAX_POT];
  double scale[5];
  // FP32 copies of the per-potential constants (rcut, truncation parameter,
  // alpha, 1/dielectric) and scalings: converting FP64 constants per pair
  // would run on the FP64 pipe.
  float fpot[YG_MAX_POT][4];
  float fscale[5];
  double *gpos[YG_MAX_POT];   // per-potential gradient, orig order (natom*3)
  double *partial;            // per block: NPOT*7 (E, Vxx, Vyy, Vzz, Vxy, Vxz, Vyz)
  int want_grad;
  int apw;                    // atoms per warp (1 .. YG_PAIR_ATOMS)
};

// Accumulator: plain (FP64 or FP32) or Kahan-compensated FP32.
template <typename T, bool KAHAN> struct Acc {
  T s;
  __device__ __forceinline__ void init() { s = (T)0; }
  __device__ __forceinline__ void add(T x) { s += x; }
  __device__ __forceinline__ double value() const { return (double)s; }
  __device__ __forceinline__ float hi() const { return (float)s; }
  __device__ __forceinline__ float lo() const { return 0.0f; }
};
template <> struct Acc<float, true> {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
  __device__ __forceinline__ float hi() const { return s; }
  __device__ __forceinline__ float lo() const { return -c; }
};

template <typename T> __device__ __forceinline__ T warp_sum(T v) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
  return v;
}

// (h, l) += (xh, xl) with an error-free TwoSum of the high parts.
__device__ __forceinline__ void two_sum_acc(float &h, float &l, float xh, float xl) {
  const float s = h + xh;
  const float bb = s - h;
  const float e = (h - (s - bb)) + (xh - bb);
  l = l + xl + e;
  h = s;
}

// Butterfly warp sum of (hi, lo) pairs; every lane ends with the total.
__device__ __forceinline__ void warp_twosum(float &h, float &l) {
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) {
    const float oh = __shfl_xor_sync(0xffffffffu, h, o);
    const float ol = __shfl_xor_sync(0xffffffffu, l, o);
    two_sum_acc(h, l, oh, ol);
  }
}

// One pair term of compile-time kind K in FP32 (mixed modes, no truncation,
// EI without Gaussian radii and with alpha > 0): the formulas and operation
// order of pair_term_f32, without its run-time dispatch.
template <int K>
__device__ __forceinline__ void pair_term_k(float alpha, float invd, float d, float inv_d, float inv_d2, float pi0,
                                            float pi1, float pi3, float pj0, float pj1, float pj3, float qi, float qj,
                                            float &v, float &g) {
  if (K == YG_POT_LJ) {
    const float sig = 0.5f * (pi0 + pj0);
    const float eps = pi1 * pj1;
    const float s2 = sig * sig * inv_d2;
    const float x = s2 * s2 * s2;
    g = 24.0f * eps * inv_d2 * x * (1.0f - 2.0f * x);
    v = 4.0f * eps * (x * (x - 1.0f));
  } else if (K == YG_POT_MM3) {
    const float sig = pi0 + pj0;
    const float eps = pi1 * pj1;
    const float inv_sig = __frcp_rn(sig);  // = 1.0f / sig (both correctly rounded)
    const float ex = 1.84e5f * expf(-12.0f * d * inv_sig);
    if (pi3 + pj3 == 0.0f) {
      const float s2 = sig * sig * inv_d2;
      const float x = 2.25f * s2 * s2 * s2;
      g = eps * inv_d * (-12.0f * inv_sig * ex + 6.0f * inv_d * x);
      v = eps * (ex - x);
    } else {
      g = eps * inv_d * (-12.0f * inv_sig * ex);
      v = eps * ex;
    }
  } else {
    const float qq = qi * qj * invd;
    const float x = alpha * d;
    const float e = expf(-x * x);
    v = qq * erfc_cheb(x) * inv_d;
    g = (-1.1283791670955126f * alpha * e * qq - v) * inv_d2;
  }
}

// One list entry of potential p (compile-time kind K) in the specialised
// mixed kernel: the term, masked with d < r_c and a nonzero scale, added to
// the potential's energy, gradient and virial sums.
template <int K, typename AccT>
__device__ __forceinline__ void pot_entry(const PairArgs &A, int p, int j, float d, float inv_d, float inv_d2, float dx,
                                          float dy, float dz, float sc, const float (&fpi)[4], float fqi, float qj,
                                          AccT &E, AccT (&G)[3], AccT (&V)[6]) {
  float pj0 = 0.f, pj1 = 0.f, pj3 = 0.f;
  if (K != YG_POT_EI) {
    const float4 q4 = *reinterpret_cast<const float4 *>(A.pp32 + (int64_t)j * 4 * YG_MAX_POT + 4 * A.pot[p].col);
    pj0 = q4.x;
    pj1 = q4.y;
    pj3 = q4.w;
  }
  float fv, fg;
  pair_term_k<K>(A.fpot[p][2], A.fpot[p][3], d, inv_d, inv_d2, fpi[0], fpi[1], fpi[3], pj0, pj1, pj3, fqi, qj, fv, fg);
  const bool in = (d < A.fpot[p][0]) && (sc != 0.0f);
  const float v = in ? fv : 0.0f;
  float g = in ? fg : 0.0f;
  const float s = in ? sc : 0.0f;
  E.add(0.5f * s * v);
  if (A.want_grad) {
    g *= s;
    G[0].add(-dx * g);
    G[1].add(-dy * g);
    G[2].add(-dz * g);
    const float hg = 0.5f * g;
    V[0].add(dx * dx * hg);
    V[1].add(dy * dy * hg);
    V[2].add(dz * dz * hg);
    V[3].add(dx * dy * hg);
    V[4].add(dx * dz * hg);
    V[5].add(dy * dz * hg);
  }
}

template <int MODE, int NPOT, int K0 = -1, int K1 = -1>
// Resident blocks per SM the specialised mixed kernel is compiled for: 3
// (79 registers, no spill) measured faster in the whole evaluation than 4 (64
// registers with a small spill): 781-784 against 768-770 evaluations/s of the
// 50,000-atom triclinic system.
#ifndef YG_PAIR_MINB
#define YG_PAIR_MINB 3
#endif
__global__ void __launch_bounds__(256, (MODE == YG_MIXED && NPOT <= 2) ? YG_PAIR_MINB : 1) k_pair(PairArgs A) {
  typedef typename std::conditional<MODE == YG_FP64, double, float>::type T;
  const bool kahan = (MODE == YG_MIXED_KAHAN);
  __shared__ double red[8][NPOT * 7];
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
  const int64_t w0 = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  Acc<T, kahan> E[NPOT], G[NPOT][3], V[NPOT][6];
#pragma unroll
  for (int p = 0; p < NPOT; p++) {
    E[p].init();
#pragma unroll
    for (int k = 0; k < 6; k++) V[p][k].init();
  }
  // A.apw atoms per warp, one after the other: each atom's gradient is
  // reduced and stored after its row; energy and virial accumulate over the
  // warp's atoms and are reduced once
  for (int ia = 0; ia < A.apw; ia++) {
  const int64_t i = w0 * A.apw + ia;
#pragma unroll
  for (int p = 0; p < NPOT; p++)
#pragma unroll
    for (int k = 0; k < 3; k++) G[p][k].init();
  if (i < A.natom) {
    T xi, yi, zi, qi;
    if (MODE == YG_FP64) {
      double4_32a x = A.x64[i];
      xi = (T)x.x; yi = (T)x.y; zi = (T)x.z; qi = (T)x.w;
    } else {
      float4 x = A.x32[i];
      xi = (T)x.x; yi = (T)x.y; zi = (T)x.z; qi = (T)x.w;
    }
    T pi[NPOT][4];
#pragma unroll
    for (int p = 0; p < NPOT; p++)
#pragma unroll
      for (int k = 0; k < 4; k++)
        pi[p][k] = (MODE == YG_FP64) ? (T)A.pp64[i * 4 * YG_MAX_POT + 4 * A.pot[p].col + k]
                                     : (T)A.pp32[i * 4 * YG_MAX_POT + 4 * A.pot[p].col + k];
    const int2 cn = A.ncount[i];
    const bool use_back = A.fresh ? (*A.fresh == 0) : (A.back != 0);
    const int cnt = cn.x + (use_back ? cn.y : 0);
    // entry e of the row: the front segment, then the back one
    const uint2 *row = A.nbr + i * A.cap;
    const uint2 *rowb = row + (A.cap - cn.y - cn.x);
    if (K0 >= 0) {
      // compile-time potential kinds (mixed modes): every term is evaluated
      // and masked with d < r_c and a nonzero scale, no per-entry dispatch
      float fpi[NPOT][4];
#pragma unroll
      for (int p = 0; p < NPOT; p++)
#pragma unroll
        for (int k = 0; k < 4; k++) fpi[p][k] = (float)pi[p][k];
      const float fxi = (float)xi, fyi = (float)yi, fzi = (float)zi, fqi = (float)qi;
      // the next entry of the lane is loaded one step ahead
      uint2 ent_next = lane < cnt ? (lane < cn.x ? row : rowb)[lane] : make_uint2(0u, 0u);
      for (int e = lane; e < cnt; e += 32) {
        const uint2 ent = ent_next;
        if (e + 32 < cnt) ent_next = (e + 32 < cn.x ? row : rowb)[e + 32];
        const int j = (int)ent.x;
        const int oidx = (int)(ent.y & YG_META_OFF_MASK);
        const int code = (int)((ent.y >> YG_META_SCALE_SHIFT) & 7u);
        const float4 xj = A.x32[j];
        const float4 sh = A.shift32[oidx];
        const float dx = (xj.x - fxi) + sh.x;
        const float dy = (xj.y - fyi) + sh.y;
        const float dz = (xj.z - fzi) + sh.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const float inv_d = rsqrtf(d2);
        const float d = d2 * inv_d;
        const float inv_d2 = inv_d * inv_d;
        const float sc = A.fscale[code];
        pot_entry<(K0 >= 0 ? K0 : 0)>(A, 0, j, d, inv_d, inv_d2, dx, dy, dz, sc, fpi[0], fqi, xj.w, E[0], G[0], V[0]);
        if (NPOT > 1)
          pot_entry<(K1 >= 0 ? K1 : 0)>(A, NPOT > 1 ? 1 : 0, j, d, inv_d, inv_d2, dx, dy, dz, sc, fpi[NPOT > 1 ? 1 : 0],
                                        fqi, xj.w, E[NPOT > 1 ? 1 : 0], G[NPOT > 1 ? 1 : 0], V[NPOT > 1 ? 1 : 0]);
      }
    }
    for (int e = (K0 >= 0) ? cnt : lane; e < cnt; e += 32) {
      const uint2 ent = (e < cn.x ? row : rowb)[e];
      const int j = (int)ent.x;
      const int oidx = (int)(ent.y & YG_META_OFF_MASK);
      const int code = (int)((ent.y >> YG_META_SCALE_SHIFT) & 7u);
      T dx, dy, dz, qj;
      if (MODE == YG_FP64) {
        double4_32a xj = A.x64[j];
        dx = (T)((xj.x - (double)xi) + A.shift64[3 * oidx]);
        dy = (T)((xj.y - (double)yi) + A.shift64[3 * oidx + 1]);
        dz = (T)((xj.z - (double)zi) + A.shift64[3 * oidx + 2]);
        qj = (T)xj.w;
      } else {
        float4 xj = A.x32[j];
        float4 sh = A.shift32[oidx];
        dx = (T)((xj.x - (float)xi) + sh.x);
        dy = (T)((xj.y - (float)yi) + sh.y);
        dz = (T)((xj.z - (float)zi) + sh.z);
        qj = (T)xj.w;
      }
      const T d2 = dx * dx + dy * dy + dz * dz;
      T d, inv_d = (T)0;
      if (MODE == YG_FP64) {
        d = Num<T>::sqrt_(d2);
      } else {
        inv_d = (T)rsqrtf((float)d2);
        d = d2 * inv_d;
      }
      const T s = (MODE == YG_FP64) ? (T)A.scale[code] : (T)A.fscale[code];
      if (s == (T)0) continue;
#pragma unroll
      for (int p = 0; p < NPOT; p++) {
        const T rcT = (MODE == YG_FP64) ? (T)A.pot[p].rcut : (T)A.fpot[p][0];
        if (!(d < rcT)) continue;
        T pj[4] = {(T)0, (T)0, (T)0, (T)0};
        if (MODE == YG_FP64) {
#pragma unroll
          for (int k = 0; k < 4; k++) pj[k] = (T)A.pp64[(int64_t)j * 4 * YG_MAX_POT + 4 * A.pot[p].col + k];
        } else if (A.pot[p].kind != YG_POT_EI || A.pot[p].has_radii) {
          const float4 q4 = *reinterpret_cast<const float4 *>(A.pp32 + (int64_t)j * 4 * YG_MAX_POT + 4 * A.pot[p].col);
          pj[0] = (T)q4.x; pj[1] = (T)q4.y; pj[2] = (T)q4.z; pj[3] = (T)q4.w;
        }
        const T parT = (MODE == YG_FP64) ? (T)A.pot[p].tr_par : (T)A.fpot[p][1];
        const T alphaT = (MODE == YG_FP64) ? (T)A.pot[p].alpha : (T)A.fpot[p][2];
        const T invdT = (MODE == YG_FP64) ? (T)A.pot[p].inv_diel : (T)A.fpot[p][3];
        T v, g;
        if (MODE == YG_FP64) {
          pair_term<T>(A.pot[p], rcT, parT, alphaT, invdT, d, d2, pi[p][0], pi[p][1], pi[p][2], pi[p][3], pj[0],
                       pj[1], pj[2], pj[3], qi, qj, v, g);
        } else {
          float fv, fg;
          pair_term_f32(A.pot[p], (float)rcT, (float)parT, (float)alphaT, (float)invdT, (float)d, (float)d2,
                        (float)inv_d, (float)pi[p][0], (float)pi[p][1], (float)pi[p][2], (float)pi[p][3],
                        (float)pj[0], (float)pj[1], (float)pj[2], (float)pj[3], (float)qi, (float)qj, fv, fg);
          v = (T)fv;
          g = (T)fg;
        }
        E[p].add((T)0.5 * s * v);
        if (A.want_grad) {
          g *= s;
          G[p][0].add(-dx * g);
          G[p][1].add(-dy * g);
          G[p][2].add(-dz * g);
          const T hg = (T)0.5 * g;
          V[p][0].add(dx * dx * hg);
          V[p][1].add(dy * dy * hg);
          V[p][2].add(dz * dz * hg);
          V[p][3].add(dx * dy * hg);
          V[p][4].add(dx * dz * hg);
          V[p][5].add(dy * dz * hg);
        }
      }
    }
  }
  // the atom's gradient
  if (A.want_grad && i < A.natom) {
    const int oi = A.sorted[i];
    if (MODE == YG_FP64) {
#pragma unroll
      for (int p = 0; p < NPOT; p++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
          const double gv = warp_sum<double>(G[p][k].value());
          if (lane == 0) A.gpos[p][3 * (int64_t)oi + k] = gv;
        }
    } else {
      float gh[NPOT * 3], gl[NPOT * 3];
#pragma unroll
      for (int p = 0; p < NPOT; p++)
#pragma unroll
        for (int k = 0; k < 3; k++) {
          gh[3 * p + k] = G[p][k].hi();
          gl[3 * p + k] = G[p][k].lo();
          warp_twosum(gh[3 * p + k], gl[3 * p + k]);
        }
      float h = gh[0], l = gl[0];
#pragma unroll
      for (int c = 1; c < NPOT * 3; c++)
        if (lane == c) {
          h = gh[c];
          l = gl[c];
        }
      if (lane < NPOT * 3) A.gpos[lane / 3][3 * (int64_t)oi + lane % 3] = (double)h + (double)l;
    }
  }
  }  // atoms of the warp
  if (MODE == YG_FP64) {
    // FP64 warp, block and grid reductions
    double part[NPOT * 7];
#pragma unroll
    for (int p = 0; p < NPOT; p++) {
      part[7 * p] = E[p].value();
#pragma unroll
      for (int k = 0; k < 6; k++) part[7 * p + 1 + k] = V[p][k].value();
    }
#pragma unroll
    for (int v = 0; v < NPOT * 7; v++) part[v] = warp_sum<double>(part[v]);
    if (lane == 0) {
#pragma unroll
      for (int v = 0; v < NPOT * 7; v++) red[wid][v] = part[v];
    }
    __syncthreads();
    if (threadIdx.x < NPOT * 7) {
      double s = 0.0;
      const int nw = blockDim.x >> 5;
      for (int w = 0; w < nw; w++) s += red[w][threadIdx.x];
      A.partial[(int64_t)blockIdx.x * NPOT * 7 + threadIdx.x] = s;
    }
  } else {
    // Mixed modes: the FP32 lane partials are combined with error-free
    // TwoSum steps into (hi, lo) FP32 pairs (about twice FP32 precision);
    // FP64 is used only where a pair becomes an FP64 result, on the few
    // lanes that store it.  A 32-lane FP64 instruction costs the GB300 FP64
    // pipe tens of cycles, so per-warp FP64 reductions would dominate.
    __shared__ float2 redf[8][NPOT * 7];
    float hi[NPOT * 7], lo[NPOT * 7];
#pragma unroll
    for (int p = 0; p < NPOT; p++) {
      hi[7 * p] = E[p].hi();
      lo[7 * p] = E[p].lo();
#pragma unroll
      for (int k = 0; k < 6; k++) {
        hi[7 * p + 1 + k] = V[p][k].hi();
        lo[7 * p + 1 + k] = V[p][k].lo();
      }
    }
#pragma unroll
    for (int v = 0; v < NPOT * 7; v++) warp_twosum(hi[v], lo[v]);
    if (lane == 0) {
#pragma unroll
      for (int v = 0; v < NPOT * 7; v++) redf[wid][v] = make_float2(hi[v], lo[v]);
    }
    __syncthreads();
    if (threadIdx.x < NPOT * 7) {
      float h = 0.0f, l = 0.0f;
      const int nw = blockDim.x >> 5;
      for (int w = 0; w < nw; w++) {
        const float2 x = redf[w][threadIdx.x];
        two_sum_acc(h, l, x.x, x.y);
      }
      A.partial[(int64_t)blockIdx.x * NPOT * 7 + threadIdx.x] = (double)h + (double)l;
    }
  }
}

// Sums column v of a (nblocks x nval) partial array in a fixed order.
__global__ void k_reduce_cols(const double *__restrict__ partials, int nblocks, int nval,
                              double *__restrict__ out) {
  __shared__ double sh[256];
  const int v = blockIdx.x;
  double s = 0.0;
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x) s += partials[(int64_t)b * nval + v];
  sh[threadIdx.x] = s;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w) sh[threadIdx.x] += sh[threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) out[v] = sh[0];
}

struct SlotMap {
  int slot[YG_MAX_POT];
};

// Writes (E, 6 virial components) of the p-th evaluated potential as the
// (E, vtens[9]) record of its result slot.
__global__ void k_store_pair_ev(const double *__restrict__ sums, int npot, SlotMap map,
                                double *__restrict__ part_ev) {
  int p = threadIdx.x;
  if (p >= npot) return;
  const double *s = sums + 7 * p;
  double *o = part_ev + 10 * (YG_PART_PAIR0 + map.slot[p]);
  o[0] = s[0];
  o[1] = s[1]; o[2] = s[4]; o[3] = s[5];
  o[4] = s[4]; o[5] = s[2]; o[6] = s[6];
  o[7] = s[5]; o[8] = s[6]; o[9] = s[3];
}

template <int MODE, int NPOT>
int launch_pair_t(yg_ctx *ctx, PairArgs &A, int nblocks) {
  k_pair<MODE, NPOT><<<nblocks, 256, 0, ctx->stream>>>(A);
  YG_LAUNCH_CHECK(ctx, "k_pair");
  return YG_OK;
}

// The mixed-precision kernel specialised on the potential kinds, for one or
// two potentials without truncation (EI without radii, alpha > 0).
template <int K0, int K1>
int launch_pair_k(yg_ctx *ctx, PairArgs &A, int nblocks) {
  if constexpr (K1 < 0) k_pair<YG_MIXED, 1, K0, K1><<<nblocks, 256, 0, ctx->stream>>>(A);
  else k_pair<YG_MIXED, 2, K0, K1><<<nblocks, 256, 0, ctx->stream>>>(A);
  YG_LAUNCH_CHECK(ctx, "k_pair");
  return YG_OK;
}

template <int K0>
int launch_pair_k1(yg_ctx *ctx, PairArgs &A, int npot, int k1, int nblocks) {
  if (npot == 1) return launch_pair_k<K0, -1>(ctx, A, nblocks);
  if (k1 == YG_POT_LJ) return launch_pair_k<K0, YG_POT_LJ>(ctx, A, nblocks);
  if (k1 == YG_POT_MM3) return launch_pair_k<K0, YG_POT_MM3>(ctx, A, nblocks);
  return launch_pair_k<K0, YG_POT_EI>(ctx, A, nblocks);
}

int launch_pair_fast(yg_ctx *ctx, PairArgs &A, int npot, int nblocks) {
  const int k0 = A.pot[0].kind, k1 = npot > 1 ? A.pot[1].kind : -1;
  if (k0 == YG_POT_LJ) return launch_pair_k1<YG_POT_LJ>(ctx, A, npot, k1, nblocks);
  if (k0 == YG_POT_MM3) return launch_pair_k1<YG_POT_MM3>(ctx, A, npot, k1, nblocks);
  return launch_pair_k1<YG_POT_EI>(ctx, A, npot, k1, nblocks);
}

template <int MODE>
int launch_pair_m(yg_ctx *ctx, PairArgs &A, int npot, int nblocks) {
  switch (npot) {
    case 1: return launch_pair_t<MODE, 1>(ctx, A, nblocks);
    case 2: return launch_pair_t<MODE, 2>(ctx, A, nblocks);
    default: return launch_pair_t<MODE, 3>(ctx, A, nblocks);
  }
}

}  // namespace

int yg_launch_reduce_ev(yg_ctx *ctx, const double *partials, int nblocks, int nval, double *out) {
  k_reduce_cols<<<nval, 256, 0, ctx->stream>>>(partials, nblocks, nval, out);
  YG_LAUNCH_CHECK(ctx, "k_reduce_cols");
  return YG_OK;
}

int yg_launch_pair(yg_ctx *ctx, int slot_mask, int want_grad) {
  PairArgs A;
  int slots[YG_MAX_POT];
  int npot = 0;
  for (int p = 0; p < YG_MAX_POT; p++) {
    if (!(slot_mask & (1 << p))) continue;
    const PairPotHost &P = ctx->pot[p];
    if (!P.active) {
      yg_set_error("pair slot not registered");
      return YG_ERR_STATE;
    }
    if (P.kind == YG_POT_EI && !ctx->have_charges) {
      yg_set_error("EI pair potential needs charges");
      return YG_ERR_STATE;
    }
    PairPotDev &D = A.pot[npot];
    D.kind = P.kind;
    D.tr_kind = P.tr_kind;
    D.rcut = P.rcut;
    D.rcut2 = P.rcut * P.rcut;
    D.tr_par = P.tr_par;
    D.alpha = P.alpha;
    D.inv_diel = 1.0 / P.dielectric;
    D.has_radii = !P.radius2.empty();
    D.col = p;
    D.ntype = P.ntype;
    D.power = P.power;
    D.tab64 = ctx->d_ptab64[p];
    D.tab32 = ctx->d_ptab32[p];
    slots[npot] = p;
    npot++;
  }
  if (npot == 0) return YG_OK;
  const int64_t N = ctx->natom;
  A.natom = N;
  A.cap = ctx->nbr_cap;
  A.nbr = ctx->d_nbr;
  A.ncount = ctx->d_ncount;
  {
    // the back segment can be skipped when no potential reaches beyond the
    // build's split and the coordinates are those the rows were built from
    bool split_ok = true;
    for (int q = 0; q < npot; q++)
      if (A.pot[q].rcut > ctx->rin_build) split_ok = false;
    A.fresh = split_ok ? ctx->pair_fresh_dev : nullptr;
    A.back = (split_ok && ctx->x_fresh) ? 0 : 1;
  }
  A.sorted = ctx->d_sorted;
  A.x64 = ctx->d_x64;
  A.x32 = ctx->d_x32;
  A.shift64 = ctx->d_shift64;
  A.shift32 = ctx->d_shift32;
  A.pp64 = ctx->d_pp64;
  A.pp32 = ctx->d_pp32;
  for (int k = 0; k < 5; k++) {
    A.scale[k] = ctx->scale_tab[k];
    A.fscale[k] = (float)ctx->scale_tab[k];
  }
  for (int q = 0; q < npot; q++) {
    A.fpot[q][0] = (float)A.pot[q].rcut;
    A.fpot[q][1] = (float)A.pot[q].tr_par;
    A.fpot[q][2] = (float)A.pot[q].alpha;
    A.fpot[q][3] = (float)A.pot[q].inv_diel;
  }
  for (int p = 0; p < YG_MAX_POT; p++) A.gpos[p] = nullptr;
  for (int q = 0; q < npot; q++) A.gpos[q] = ctx->d_part_gpos + (size_t)(YG_PART_PAIR0 + slots[q]) * N * 3;
  A.want_grad = want_grad;
  SlotMap map;
  for (int q = 0; q < YG_MAX_POT; q++) map.slot[q] = q < npot ? slots[q] : 0;
  // atoms per warp: the most (up to YG_PAIR_ATOMS) that still leaves at
  // least two full waves of warps (4 blocks of 8 warps per SM), so that a
  // small system keeps the machine busy to the end
  A.apw = 1;
  while (2 * A.apw <= YG_PAIR_ATOMS && (N / (2 * A.apw)) >= (int64_t)2 * ctx->nsm * 32) A.apw *= 2;
  const int nblocks = yg_blocks((N + A.apw - 1) / A.apw * 32, 256);
  const int nval = npot * 7;
  int rc;
  if ((rc = yg_ensure(ctx, (void **)&ctx->d_red, &ctx->red_cap,
                      ((size_t)nblocks * nval + 64 + nval) * sizeof(double))))
    return rc;
  A.partial = ctx->d_red + 64;
  bool fast = ctx->precision == YG_MIXED && npot <= 2;
  for (int q = 0; q < npot; q++) {
    const PairPotDev &D = A.pot[q];
    if (D.tr_kind != YG_TR_NONE || (D.kind != YG_POT_LJ && D.kind != YG_POT_MM3 && D.kind != YG_POT_EI) ||
        (D.kind == YG_POT_EI && (D.has_radii || !(D.alpha > 0.0))))
      fast = false;
  }
  if (ctx->precision == YG_FP64) rc = launch_pair_m<YG_FP64>(ctx, A, npot, nblocks);
  else if (fast) rc = launch_pair_fast(ctx, A, npot, nblocks);
  else if (ctx->precision == YG_MIXED) rc = launch_pair_m<YG_MIXED>(ctx, A, npot, nblocks);
  else rc = launch_pair_m<YG_MIXED_KAHAN>(ctx, A, npot, nblocks);
  if (rc) return rc;
  double *sums = ctx->d_red + 64 + (size_t)nblocks * nval;
  if ((rc = yg_launch_reduce_ev(ctx, A.partial, nblocks, nval, sums))) return rc;
  k_store_pair_ev<<<1, 32, 0, ctx->stream>>>(sums, npot, map, ctx->d_part_ev);
  YG_LAUNCH_CHECK(ctx, "k_store_pair_ev");
  if (!want_grad) {
    for (int q = 0; q < npot; q++)
      YG_CUDA(cudaMemsetAsync(ctx->d_part_gpos + (size_t)(YG_PART_PAIR0 + slots[q]) * N * 3, 0,
                              N * 3 * sizeof(double), ctx->stream));
  }
  for (int q = 0; q < npot; q++) ctx->part_valid[YG_PART_PAIR0 + slots[q]] = 1;
  return YG_OK;
}
