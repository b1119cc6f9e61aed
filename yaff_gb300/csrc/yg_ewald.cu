// yg_ewald.cu -- kernel (c): Ewald reciprocal-space sum and its corrections.
//
// Same half-sphere direct sum as yaff/pes/ewald.c:32-150, restructured for
// the GPU.  Write the phase of atom a at k = 2 pi (g0 b0 + g1 b1 + m b2) as
// E0[a][g0] E1[a][g1] E2[a][m] with Ei[a][g] = exp(2 pi i g s_ai) (s = the
// fractional coordinates; negative g by conjugation).  Then
//
//   S[c][m] = sum_a X[a][c] Y[a][m],  X = E0 E1 (column c = (g0, g1)),
//                                     Y = q E2
//
// is a complex matrix product over the atoms, and the gradient
//
//   dE/dr_a = -2 pi (b0 sum_c g0 Im(P_ac Z_ac) + b1 sum_c g1 Im(P_ac Z_ac)
//                     + b2 sum_c Im(P_ac Z2_ac)),
//   Z_ac = sum_m Y[a][m] conj(W[c][m]),  Z2_ac = sum_m m Y[a][m] conj(W[c][m]),
//   P_ac = X[a][c],  W = 2 A(k) S_eff(k)
//
// is a second product over m.  Both run as shared-memory tiled kernels over
// tiles of (g0, g1) columns sorted by their extent in m inside the k-sphere,
// so each tile loops only over the m values it needs.  The phases are built per atom from FP64 fractional coordinates
// (reduced to [0,1) before the sine/cosine), so FP32 tables keep ~1e-7
// absolute phase accuracy even where |k.r| reaches hundreds of radians.
// Partial structure factors of atom chunks are summed in FP64 in a fixed
// order; the energy, the virial and the prefactors are FP64.
#include <algorithm>
#include <utility>
#include <cmath>
#include <type_traits>
#include <mutex>
#include <set>
#include <vector>

#include <cuda_fp16.h>

#include "yg_internal.cuh"

namespace {

#define EW_SC 128    // columns per S-pass tile
#ifndef YG_UMMA_SETUP
#define YG_UMMA_SETUP 20.0  // tcgen05 force pass: a CTA's set-up cost in tile-equivalents (range choice)
#endif
#define EW_FC 64     // columns per force-pass tile
#define EW_MS 32     // m values per S-pass slab
#define EW_MAXM 64   // largest supported G2 + 1
#define EW_FEPI 3    // force-pass cost of a column tile's epilogue, in m iterations
#ifndef YG_FORCE_MINB
#define YG_FORCE_MINB 3  // resident FP32 force-pass blocks per SM the register budget is sized for
#endif

// Row stride of the per-atom phase tables: the logical length G0+G1+G2+3
// rounded up to an even count, so rows of FP32 complex values are whole
// 16-byte units (bulk-copy granularity).
__host__ __device__ __forceinline__ int ew_row_stride(int G0, int G1, int G2) { return (G0 + G1 + G2 + 4) & ~1; }


template <typename T> struct C2;
template <> struct C2<float> { typedef float2 t; };
template <> struct C2<double> { typedef double2 t; };

template <typename T> __device__ __forceinline__ typename C2<T>::t cmk(T a, T b) {
  typename C2<T>::t r;
  r.x = a;
  r.y = b;
  return r;
}

// Per-atom phase tables: for every atom L = (G0+1)+(G1+1)+(G2+1) complex
// values, E0[0..G0], E1[0..G1], q*E2[0..G2].
// One thread per (atom, axis): the fractional coordinate s is formed once in
// FP64; every entry's argument g*s mod 1 is then reduced exactly -- in FP64
// for the plain form, and for the FP32 forms from the split s = s_hi + s_lo
// with the exact product error fmaf(g, s_hi, -g*s_hi) -- before the FP32 or
// FP64 sine/cosine.
template <typename T>
__global__ void k_tables(const double *__restrict__ pos, const double *__restrict__ charge, int64_t natom,
                         CellGeom cell, int G0, int G1, int G2, typename C2<T>::t *__restrict__ tab) {
  const int L = ew_row_stride(G0, G1, G2);
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= natom * 3) return;
  const int64_t a = idx / 3;
  const int axis = (int)(idx - a * 3);
  const int gmax = axis == 0 ? G0 : (axis == 1 ? G1 : G2);
  const int base = axis == 0 ? 0 : (axis == 1 ? G0 + 1 : G0 + G1 + 2);
  const double *gv = cell.gv + 3 * axis;
  double s = gv[0] * pos[3 * a] + gv[1] * pos[3 * a + 1] + gv[2] * pos[3 * a + 2];
  s -= floor(s);
  const T q = (axis == 2) ? (T)charge[a] : (T)1;
  typename C2<T>::t *out = tab + a * L + base;
  if (sizeof(T) == 8) {
    for (int g = 0; g <= gmax; g++) {
      double x = (double)g * s;
      x -= rint(x);
      double dsn, dcs;
      sincospi(2.0 * x, &dsn, &dcs);
      out[g] = cmk<T>((T)dcs * q, (T)dsn * q);
    }
  } else {
    const float s_hi = (float)s;
    const float s_lo = (float)(s - (double)s_hi);
    for (int g = 0; g <= gmax; g++) {
      const float fg = (float)g;
      const float p = fg * s_hi;
      const float e = fmaf(fg, s_hi, -p);
      const float x = (p - rintf(p)) + fmaf(fg, s_lo, e);
      float fsn, fcs;
      sincospif(2.0f * x, &fsn, &fcs);
      out[g] = cmk<T>((T)fcs * q, (T)fsn * q);
    }
  }
}

template <typename T>
__device__ __forceinline__ typename C2<T>::t tab_get(const typename C2<T>::t *__restrict__ row, int base, int g) {
  typename C2<T>::t v = row[base + (g < 0 ? -g : g)];
  if (g < 0) v.y = -v.y;
  return v;
}

// Sorted column descriptors: (g0, g1, dense column index, mhi), ordered by
// decreasing mhi (the largest m of the column inside the half sphere) and
// padded with (0, 0, -1, -1) to a multiple of EW_SC.  Grouping columns of
// similar extent keeps the per-tile m range tight.

// acc += x y (complex).  FP32: two packed f32x2 FMAs,
// acc += (xr, xr) (yr, yi) and acc += (-xi, xi) (yi, yr), half the issue
// slots of four scalar FMAs; FP64: scalar.
__device__ __forceinline__ void cmac(float2 &acc, float2 x, float2 y) {
  acc = __ffma2_rn(make_float2(x.x, x.x), y, acc);
  acc = __ffma2_rn(make_float2(-x.y, x.y), make_float2(y.y, y.x), acc);
}
__device__ __forceinline__ void cmac(double2 &acc, double2 x, double2 y) {
  acc.x += x.x * y.x - x.y * y.y;
  acc.y += x.x * y.y + x.y * y.x;
}

template <typename T> struct SfacCfg;
template <> struct SfacCfg<float> { enum { KA = 32, ATB = 512 }; };
template <> struct SfacCfg<double> { enum { KA = 16, ATB = 256 }; };

// ---- bulk copies into shared memory completed on an mbarrier ----
__device__ __forceinline__ unsigned smem_u32(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

__device__ __forceinline__ void mbar_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(smem_u32(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ void mbar_init_fence() {
  asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
}

// The barrier's single arrival, announcing `bytes` of copies to come.
__device__ __forceinline__ void bulk_expect(unsigned long long *bar, unsigned bytes) {
  unsigned long long state;  // arrival token (unused: waits go by phase parity)
  asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
               : "=l"(state)
               : "r"(smem_u32(bar)), "r"(bytes)
               : "memory");
}

// Copy of `bytes` (a multiple of 16, both addresses 16-byte aligned) from
// global into shared memory, completing on the barrier.
__device__ __forceinline__ void bulk_copy(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   smem_u32(dst)),
               "l"(src), "r"(bytes), "r"(smem_u32(bar))
               : "memory");
}

__device__ __forceinline__ void bulk_load(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  bulk_expect(bar, bytes);
  bulk_copy(dst, src, bytes, bar);
}

// Waits for phase `parity` of the barrier; gives up after a bounded number
// of polls (about a second), records the failure and returns false.
__device__ __forceinline__ bool mbar_wait(unsigned long long *bar, unsigned parity, int *status) {
  for (int it = 0; it < (1 << 24); it++) {
    unsigned ok;
    asm volatile(
        "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
        : "=r"(ok)
        : "r"(smem_u32(bar)), "r"(parity)
        : "memory");
    if (ok) return true;
  }
  if (status) atomicOr(status + YG_ST_TIMEOUT, 1);
  return false;
}

// The S-pass MACs of one warp over the staged rows of a chunk: columns are
// formed as X = E0 E1 (conjugated for negative g0, g1; zero for padding
// columns) and acc[i][j] += X_i Y_j for the warp's nj m values.  FP32 takes
// nj as the compile-time count NJ, so the m loop is straight-line code whose
// shared loads the compiler issues ahead of the FMAs; FP64 (NJ == 0, twice
// the registers per value) keeps a run-time count.
template <typename T, int NJ>
__device__ __forceinline__ void sfac_rows(const typename C2<T>::t *__restrict__ buf, int nrow, int L,
                                          const int (&o0)[4], const int (&o1)[4], const T (&s0)[4],
                                          const T (&s1)[4], const T (&ok)[4], int yb, int nj,
                                          typename C2<T>::t (&acc)[4][8]) {
  typedef typename C2<T>::t CT;
  const int NY = NJ > 0 ? NJ : 1;
#pragma unroll(NJ > 0 ? 1 : 2)
  for (int la = 0; la < nrow; la++) {
    const CT *row = buf + la * L;
    CT y[NY];
    if (NJ > 0) {
#pragma unroll
      for (int j = 0; j < NY; j++) y[j] = row[yb + 4 * j];
    }
    CT x[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      CT e0 = row[o0[i]], e1 = row[o1[i]];
      e0.x *= ok[i];
      e0.y *= s0[i] * ok[i];
      e1.y *= s1[i];
      x[i] = cmk<T>(e0.x * e1.x - e0.y * e1.y, e0.x * e1.y + e0.y * e1.x);
    }
    if (NJ > 0) {
#pragma unroll
      for (int j = 0; j < NY; j++)
#pragma unroll
        for (int i = 0; i < 4; i++) cmac(acc[i][j], x[i], y[j]);
    } else {
#pragma unroll
      for (int j = 0; j < 8; j++) {
        if (j < nj) {
          const CT yj = row[yb + 4 * j];
#pragma unroll
          for (int i = 0; i < 4; i++) cmac(acc[i][j], x[i], yj);
        }
      }
    }
  }
}

// S pass.  grid = (atom chunks, column tiles, m slabs), 128 threads = 4 warps:
// blocks start in tile-major order, the tiles sorted by decreasing extent,
// so the short blocks of the last tiles fill the tail of the launch.
// The table rows of KA atoms are staged in shared memory with coalesced
// copies.  Lane l owns columns l, l+32, l+64, l+96 of the tile and forms
// X = E0 E1 for them from the staged rows; warp w owns m = w + 4j, j < 8,
// of the slab (broadcast loads of Y), so m values beyond the tile's extent
// are skipped warp-uniformly.
template <typename T, typename TA>
__global__ void __launch_bounds__(128) k_sfac(const typename C2<T>::t *__restrict__ tab, int a0, int a1, int G0,
                                              int G1, int G2, const int4 *__restrict__ cols,
                                              typename C2<TA>::t *__restrict__ Spart, int nstile, int nslab,
                                              int *__restrict__ status) {
  typedef typename C2<T>::t CT;
  const int KA = SfacCfg<T>::KA, ATB = SfacCfg<T>::ATB;
  const int L = ew_row_stride(G0, G1, G2);
  extern __shared__ __align__(16) unsigned char sfac_smem[];
  __shared__ unsigned long long bars[2];
  CT *sRow = reinterpret_cast<CT *>(sfac_smem);      // 2 x [KA][L] table rows
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int tile = blockIdx.y, slab = blockIdx.z;
  const int mb = slab * EW_MS;
  const int Mt = cols[tile * EW_SC].w + 1 - mb;
  const int nj = (Mt > w) ? min(8, (Mt - w + 3) / 4) : 0;
  const int abeg = a0 + blockIdx.x * ATB;
  const int aend = min(a1, abeg + ATB);
  CT acc[4][8];
#pragma unroll
  for (int i = 0; i < 4; i++)
#pragma unroll
    for (int j = 0; j < 8; j++) acc[i][j] = cmk<T>((T)0, (T)0);
  if (Mt > 0 && aend > abeg) {
    int o0[4], o1[4];
    T s0[4], s1[4], ok[4];
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int4 col = cols[tile * EW_SC + lane + 32 * i];
      o0[i] = col.x < 0 ? -col.x : col.x;
      o1[i] = G0 + 1 + (col.y < 0 ? -col.y : col.y);
      s0[i] = col.x < 0 ? (T)-1 : (T)1;
      s1[i] = col.y < 0 ? (T)-1 : (T)1;
      ok[i] = col.z >= 0 ? (T)1 : (T)0;
    }
    const int yb = G0 + G1 + 2 + mb + w;
    // the chunks' table rows are contiguous in global memory: double-buffered
    // bulk copies, the next chunk in flight while this one is consumed
    const int nchunk = (aend - abeg + KA - 1) / KA;
    if (threadIdx.x == 0) {
      mbar_init(&bars[0], 1);
      mbar_init(&bars[1], 1);
      mbar_init_fence();
    }
    __syncthreads();
    if (threadIdx.x == 0) {
      const int nrow = min(KA, aend - abeg);
      bulk_load(sRow, tab + (int64_t)abeg * L, (unsigned)(nrow * L * sizeof(CT)), &bars[0]);
    }
    for (int c = 0; c < nchunk; c++) {
      const int ab = abeg + c * KA;
      const int nrow = min(KA, aend - ab);
      if (threadIdx.x == 0 && c + 1 < nchunk) {
        const int ab1 = ab + KA;
        bulk_load(sRow + (size_t)((c + 1) & 1) * KA * L, tab + (int64_t)ab1 * L,
                  (unsigned)(min(KA, aend - ab1) * L * sizeof(CT)), &bars[(c + 1) & 1]);
      }
      const bool arrived = mbar_wait(&bars[c & 1], (unsigned)((c >> 1) & 1), status);
      if (__syncthreads_or(!arrived)) {
        // a copy never completed: wait (bounded) for the one still in flight
        if (threadIdx.x == 0 && c + 1 < nchunk) mbar_wait(&bars[(c + 1) & 1], (unsigned)(((c + 1) >> 1) & 1), status);
        break;
      }
      const CT *buf = sRow + (size_t)(c & 1) * KA * L;
      if (sizeof(T) == 8) {
        sfac_rows<T, 0>(buf, nrow, L, o0, o1, s0, s1, ok, yb, nj, acc);
      } else {
        // nj is warp-uniform: one branch per chunk selects a straight-line body
        switch (nj) {
          case 8: sfac_rows<T, 8>(buf, nrow, L, o0, o1, s0, s1, ok, yb, nj, acc); break;
          case 7: sfac_rows<T, 7>(buf, nrow, L, o0, o1, s0, s1, ok, yb, nj, acc); break;
          case 6: sfac_rows<T, 6>(buf, nrow, L, o0, o1, s0, s1, ok, yb, nj, acc); break;
          case 5: sfac_rows<T, 5>(buf, nrow, L, o0, o1, s0, s1, ok, yb, nj, acc); break;
          case 4: sfac_rows<T, 4>(buf, nrow, L, o0, o1, s0, s1, ok, yb, nj, acc); break;
          case 3: sfac_rows<T, 3>(buf, nrow, L, o0, o1, s0, s1, ok, yb, nj, acc); break;
          case 2: sfac_rows<T, 2>(buf, nrow, L, o0, o1, s0, s1, ok, yb, nj, acc); break;
          case 1: sfac_rows<T, 1>(buf, nrow, L, o0, o1, s0, s1, ok, yb, nj, acc); break;
          default: break;
        }
      }
      __syncthreads();  // every thread is done with this buffer before it is refilled
    }
  }
  // partial layout: [chunk][tile][slab][c][m]
  typedef typename C2<TA>::t CA;
  const int64_t base = (((int64_t)blockIdx.x * nstile + tile) * nslab + slab) * (EW_SC * EW_MS);
#pragma unroll
  for (int i = 0; i < 4; i++) {
    const int c = lane + 32 * i;
#pragma unroll
    for (int j = 0; j < 8; j++) {
      CA v;
      v.x = (TA)acc[i][j].x;
      v.y = (TA)acc[i][j].y;
      Spart[base + c * EW_MS + w + 4 * j] = v;
    }
  }
}

// Sums the chunk partials in a fixed order into the dense S[col][m]: four
// threads per element each sum every fourth chunk (FP64, or error-free
// TwoSum (hi, lo) pairs of the FP32 partials), then the four sums are
// combined by a fixed butterfly within the aligned group of four lanes.
__device__ __forceinline__ void two_sum_f(float &h, float &l, float xh, float xl) {
  const float s = h + xh, bb = s - h;
  l += (h - (s - bb)) + (xh - bb) + xl;
  h = s;
}

template <typename TA>
__global__ void k_sfac_reduce(const typename C2<TA>::t *__restrict__ Spart, int nchunk, int nstile, int nslab, int sc,
                              const int4 *__restrict__ cols, int nm, double unscale, double *__restrict__ S) {
  const int64_t tid = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t idx = tid >> 2;
  const int sub = (int)(tid & 3);
  const int64_t per = (int64_t)nstile * nslab * sc * EW_MS;
  if (idx >= per) return;  // whole groups of four leave together (per-group condition)
  const int m = (int)(idx % EW_MS);
  const int c = (int)((idx / EW_MS) % sc);
  const int slab = (int)((idx / (EW_MS * sc)) % nslab);
  const int tile = (int)(idx / ((int64_t)EW_MS * sc * nslab));
  const int4 col = cols[tile * sc + c];
  const int mm = slab * EW_MS + m;
  if (col.z < 0 || mm > col.w) return;
  const unsigned gmask = 0xFu << (threadIdx.x & 28);
  double re, im;
  if (sizeof(TA) == 8) {
    re = 0.0;
    im = 0.0;
    for (int ch = sub; ch < nchunk; ch += 4) {
      const typename C2<TA>::t v = Spart[(int64_t)ch * per + idx];
      re += (double)v.x;
      im += (double)v.y;
    }
    re += __shfl_xor_sync(gmask, re, 1);
    im += __shfl_xor_sync(gmask, im, 1);
    re += __shfl_xor_sync(gmask, re, 2);
    im += __shfl_xor_sync(gmask, im, 2);
  } else {
    // FP32 partials: (hi, lo) pairs, one conversion to FP64 at the end (the
    // FP64 pipe is the slow one)
    float rh = 0.f, rl = 0.f, ih = 0.f, il = 0.f;
    for (int ch = sub; ch < nchunk; ch += 4) {
      const typename C2<TA>::t v = Spart[(int64_t)ch * per + idx];
      two_sum_f(rh, rl, (float)v.x, 0.f);
      two_sum_f(ih, il, (float)v.y, 0.f);
    }
#pragma unroll
    for (int o = 1; o <= 2; o <<= 1) {
      const float orh = __shfl_xor_sync(gmask, rh, o), orl = __shfl_xor_sync(gmask, rl, o);
      const float oih = __shfl_xor_sync(gmask, ih, o), oil = __shfl_xor_sync(gmask, il, o);
      // both lanes of a pair add in the same order: lower lane's value first
      if (sub & o) {
        float h = orh, l = orl;
        two_sum_f(h, l, rh, rl);
        rh = h;
        rl = l;
        h = oih;
        l = oil;
        two_sum_f(h, l, ih, il);
        ih = h;
        il = l;
      } else {
        two_sum_f(rh, rl, orh, orl);
        two_sum_f(ih, il, oih, oil);
      }
    }
    re = (double)rh + (double)rl;
    im = (double)ih + (double)il;
  }
  if (sub == 0) {
    S[2 * ((int64_t)col.z * nm + mm)] = re * unscale;
    S[2 * ((int64_t)col.z * nm + mm) + 1] = im * unscale;
  }
}

// FP16 split of a weight pair into the force pass's B fragments (see the
// tensor-core section below); record words: hi b0, hi b1, lo b0, lo b1.
__device__ __forceinline__ void wb_put(unsigned *__restrict__ rec, int bsel, int off, float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  const float2 f = __half22float2(h);
  const __half2 l = __floats2half2_rn(a - f.x, b - f.y);
  rec[off + bsel] = *reinterpret_cast<const unsigned *>(&h);
  rec[off + 2 + bsel] = *reinterpret_cast<const unsigned *>(&l);
}

// FP16 split of a weight pair into a B-operand unit of the tcgen05 force
// pass: hi at word w of the unit's first 8 KB, lo at the same word of the
// second.
__device__ __forceinline__ void ub_put(unsigned *__restrict__ unit, int w, float a, float b) {
  const __half2 h = __floats2half2_rn(a, b);
  const float2 f = __half22float2(h);
  const __half2 l = __floats2half2_rn(a - f.x, b - f.y);
  unit[w] = *reinterpret_cast<const unsigned *>(&h);
  unit[w + 2048] = *reinterpret_cast<const unsigned *>(&l);
}

template <typename T>
__global__ void k_ewald_energy(const double *__restrict__ S, int nS, int64_t nk_dense, const double *__restrict__ pref,
                               int G0, int G1, int nm, CellGeom cell, double fac2, int ngroup,
                               const int *__restrict__ wslot, int64_t wstride, typename C2<T>::t *__restrict__ W,
                               unsigned *__restrict__ wbw, const int *__restrict__ woff, int64_t wbstride,
                               unsigned *__restrict__ ubw, const int *__restrict__ uoff, int64_t ubstride,
                               const int *__restrict__ uslot,
                               double wsc1, double wsc2, double *__restrict__ partial) {
  __shared__ double red[256 / 32][7];
  int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double e = 0.0, v[6] = {0, 0, 0, 0, 0, 0};
  if (idx < nk_dense) {
    double A = pref[idx];
    const double *S0 = S + 2 * idx;
    double c0 = S0[0], s0 = S0[1], c1 = 0, s1 = 0, c2 = 0, s2 = 0;
    if (nS == 3) {
      c1 = S[2 * (nk_dense + idx)];
      s1 = S[2 * (nk_dense + idx) + 1];
      c2 = S[2 * (2 * nk_dense + idx)];
      s2 = S[2 * (2 * nk_dense + idx) + 1];
    }
    if (A != 0.0) {
      double s = c0 * (c0 + 2.0 * (c1 + c2)) + s0 * (s0 + 2.0 * (s1 + s2));
      s += 2.0 * (c1 * c2 + s1 * s2);
      e = A * s;
      int64_t col = idx / nm;
      int m = (int)(idx - col * nm);
      int g0 = (int)(col / (2 * G1 + 1)) - G0;
      int g1 = (int)(col % (2 * G1 + 1)) - G1;
      double k[3];
      const double tp = 6.2831853071795864769;
      for (int x = 0; x < 3; x++)
        k[x] = tp * (g0 * cell.gv[x] + g1 * cell.gv[3 + x] + m * cell.gv[6 + x]);
      double ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
      double cc = A * 2.0 * (1.0 / ksq + fac2) * s;
      v[0] = cc * k[0] * k[0];
      v[1] = cc * k[1] * k[1];
      v[2] = cc * k[2] * k[2];
      v[3] = cc * k[0] * k[1];
      v[4] = cc * k[0] * k[2];
      v[5] = cc * k[1] * k[2];
    }
    // weights: group 0 = mid atoms (S0+S1+S2), 1 = low atoms (S0+S2),
    // 2 = high atoms (S0+S1); conj stored.
    const int64_t colx = idx / nm;
    const int slot = wslot[colx];
    if (slot >= 0) {
      const int mm = (int)(idx - colx * nm);
      const int64_t wpos = ((int64_t)(slot / EW_FC) * nm + mm) * EW_FC + (slot % EW_FC);
      for (int g = 0; g < ngroup; g++) {
        double wr = c0, wi = s0;
        if (g == 0) { wr += c1 + c2; wi += s1 + s2; }
        else if (g == 1) { wr += c2; wi += s2; }
        else { wr += c1; wi += s1; }
        const double ur = 2.0 * A * wr, ui = -2.0 * A * wi;  // U = conj(2 A S_eff)
        if (W) W[(int64_t)g * wstride + wpos] = cmk<T>((T)ur, (T)ui);
        const int ft = slot >> 2, ks = mm >> 3;
        if (wbw && ks < woff[ft + 1] - woff[ft]) {  // m values past the tile's extent have no unit
          // B[(m, re)][(c, re)] = Ur, B[(m, im)][(c, re)] = -Ui, B[(m, re)][(c, im)] = Ui,
          // B[(m, im)][(c, im)] = Ur; lane 4 (2 cq + q) + (m & 3), b0 for m & 7 < 4
          const int cq = slot & 3, ml = mm & 7;
          const int bsel = ml >> 2;
          // unit: the 32 lanes' Z records (4 words each), then their Z2 records
          unsigned *unit = wbw + (int64_t)g * wbstride + (int64_t)(woff[ft] + ks) * 256;
          unsigned *rq0 = unit + (4 * (2 * cq) + (ml & 3)) * 4;
          unsigned *rq1 = unit + (4 * (2 * cq + 1) + (ml & 3)) * 4;
          const double a1 = wsc1, a2 = wsc2 * mm;  // weight scales of Z and Z2
          wb_put(rq0, bsel, 0, (float)(a1 * ur), (float)(-a1 * ui));
          wb_put(rq1, bsel, 0, (float)(a1 * ui), (float)(a1 * ur));
          wb_put(rq0 + 128, bsel, 0, (float)(a2 * ur), (float)(-a2 * ui));
          wb_put(rq1 + 128, bsel, 0, (float)(a2 * ui), (float)(a2 * ur));
        }
        // the tcgen05 force pass's own tile list (conjugate pairs) places the column at us
        const int us = ubw ? uslot[colx] : -1;
        const int ut = us >> 6, uks = mm >> 3;
        if (ubw && us >= 0 && uks < uoff[ut + 1] - uoff[ut]) {
          // tcgen05 B operand: row n = 4 j + q of the tile (q: Z re, Z im,
          // Z2 re, Z2 im), K element 2 ml + (re, im) of m = 8 ks + ml; in the
          // no-swizzle K-major layout the (re, im) pair is one 32-bit word
          unsigned *unit = ubw + (int64_t)g * ubstride + (int64_t)(uoff[ut] + uks) * 4096;
          const int j = us & 63, ml = mm & 7;
          const double a1 = wsc1, a2 = wsc2 * mm;
          const int wb0 = (ml >> 2) * 32 + (ml & 3);
          const int n0 = 4 * j;
          ub_put(unit, ((n0 + 0) >> 3) * 64 + ((n0 + 0) & 7) * 4 + wb0, (float)(a1 * ur), (float)(-a1 * ui));
          ub_put(unit, ((n0 + 1) >> 3) * 64 + ((n0 + 1) & 7) * 4 + wb0, (float)(a1 * ui), (float)(a1 * ur));
          ub_put(unit, ((n0 + 2) >> 3) * 64 + ((n0 + 2) & 7) * 4 + wb0, (float)(a2 * ur), (float)(-a2 * ui));
          ub_put(unit, ((n0 + 3) >> 3) * 64 + ((n0 + 3) & 7) * 4 + wb0, (float)(a2 * ui), (float)(a2 * ur));
        }
      }
    }
  }
  // block reduction (fixed order)
  double vals[7] = {e, v[0], v[1], v[2], v[3], v[4], v[5]};
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 7; q++) {
    double x = vals[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    vals[q] = x;
  }
  if (lane == 0)
    for (int q = 0; q < 7; q++) red[wid][q] = vals[q];
  __syncthreads();
  if (threadIdx.x < 7) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w][threadIdx.x];
    partial[(int64_t)blockIdx.x * 7 + threadIdx.x] = s;
  }
}

template <typename T> struct CompAcc {
  T s;
  __device__ __forceinline__ void init() { s = (T)0; }
  __device__ __forceinline__ void add(T x) { s += x; }
  __device__ __forceinline__ double value() const { return (double)s; }
};
template <> struct CompAcc<float> {
  float s, c;
  __device__ __forceinline__ void init() { s = 0.f; c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    float y = x - c;
    float t = s + y;
    c = (t - s) - y;
    s = t;
  }
  __device__ __forceinline__ double value() const { return (double)s - (double)c; }
};

// Force pass.  One block per atom tile (16*RA atoms) of one group, over all
// column tiles -- except the tiles of the launch's last, partial wave, which
// are split into `nsplit` blocks over column ranges of equal cost (fpre =
// prefix sums of the column tiles' costs) so that the last wave is as full
// as the others; those blocks write their sums to pieces
// [tile - nfull][part][NA][3] that k_ewald_force_combine adds in order.
// 256 threads: ta = tid % 16 owns atoms ta + 16 r (r < RA), tc = tid / 16
// owns columns 4 tc .. 4 tc + 3 of each 64-column tile (shared loads of Y
// are contiguous across lanes, loads of W broadcast).  Tiles follow the
// sorted column list, so the m loop of a tile stops at its extent.
__device__ __forceinline__ int split_cut(const int *__restrict__ fpre, int nftile, int part, int nsplit) {
  // first column tile whose prefix cost reaches part/nsplit of the total
  const long long want = (long long)fpre[nftile] * part;
  int lo = 0, hi = nftile;
  while (lo < hi) {
    const int mid = (lo + hi) >> 1;
    if ((long long)fpre[mid] * nsplit >= want) hi = mid;
    else lo = mid + 1;
  }
  return lo;
}

template <typename T, int RA>
__global__ void __launch_bounds__(256, sizeof(T) == 4 ? YG_FORCE_MINB : 1) k_ewald_force(const typename C2<T>::t *__restrict__ tab, int a0, int a1,
                                                     int G0, int G1, int G2, const int4 *__restrict__ cols,
                                                     int nftile, const int *__restrict__ fpre, int nfull,
                                                     int nsplit, const typename C2<T>::t *__restrict__ Wt,
                                                     double *__restrict__ gfrac, double *__restrict__ piece,
                                                     int *__restrict__ status) {
  typedef typename C2<T>::t CT;
  extern __shared__ __align__(16) unsigned char smem_raw[];
  __shared__ unsigned long long bars[2];
  const int NA = 16 * RA;
  const int nm = G2 + 1;
  const int L = ew_row_stride(G0, G1, G2);
  const int LE = G0 + G1 + 2;                          // E0 and E1 entries of a row
  const int LEs = LE | 1;  // odd row stride: the 16 rows one load touches fall in distinct banks
  CT *sY = reinterpret_cast<CT *>(smem_raw);          // [nm][NA]
  CT *sE = sY + (size_t)nm * NA;                       // [NA][LEs]
  CT *sWb = sE + (size_t)NA * LEs;                     // 2 x [nm][EW_FC]
  int4 *scolb = reinterpret_cast<int4 *>(sWb + (size_t)2 * nm * EW_FC);  // 2 x [EW_FC]
  const int ta = threadIdx.x & 15, tc = threadIdx.x >> 4;
  int atile, ct0 = 0, ct1 = nftile, part = -1;
  if ((int)blockIdx.x < nfull) {
    atile = blockIdx.x;
  } else {
    const int idx = blockIdx.x - nfull;
    atile = nfull + idx / nsplit;
    part = idx % nsplit;
    ct0 = split_cut(fpre, nftile, part, nsplit);
    ct1 = split_cut(fpre, nftile, part + 1, nsplit);
  }
  const int abase = a0 + atile * NA;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init_fence();
  }
  for (int v = threadIdx.x; v < nm * NA; v += blockDim.x) {
    const int m = v / NA, la = v % NA;
    const int a = abase + la;
    sY[v] = (a < a1) ? tab[(int64_t)a * L + G0 + G1 + 2 + m] : cmk<T>((T)0, (T)0);
  }
  for (int v = threadIdx.x; v < NA * LE; v += blockDim.x) {
    const int la = v / LE, e = v % LE;
    const int a = abase + la;
    sE[la * LEs + e] = (a < a1) ? tab[(int64_t)a * L + e] : cmk<T>((T)0, (T)0);
  }
  __syncthreads();
  // column tiles (weights tile-ordered: [m][EW_FC], plus the 64 column
  // descriptors) through double-buffered bulk copies
  auto issue = [&](int t, int k) {
    const int4 *tcols = cols + t * EW_FC;
    const int Mt = tcols[0].w + 1;
    const unsigned wbytes = (unsigned)(Mt * EW_FC * sizeof(CT));
    const unsigned cbytes = (unsigned)(EW_FC * sizeof(int4));
    unsigned long long *bar = &bars[k & 1];
    bulk_expect(bar, wbytes + cbytes);
    bulk_copy(sWb + (size_t)(k & 1) * nm * EW_FC, Wt + (size_t)t * nm * EW_FC, wbytes, bar);
    bulk_copy(scolb + (k & 1) * EW_FC, tcols, cbytes, bar);
  };
  if (threadIdx.x == 0 && ct1 > ct0) issue(ct0, 0);
  CompAcc<T> acc[RA][3];
#pragma unroll
  for (int r = 0; r < RA; r++)
#pragma unroll
    for (int q = 0; q < 3; q++) acc[r][q].init();
  for (int t = ct0; t < ct1; t++) {
    const int k = t - ct0;  // buffer k & 1, phase (k >> 1) & 1
    if (threadIdx.x == 0 && t + 1 < ct1) issue(t + 1, k + 1);
    const bool arrived = mbar_wait(&bars[k & 1], (unsigned)((k >> 1) & 1), status);
    if (__syncthreads_or(!arrived)) {
      if (threadIdx.x == 0 && t + 1 < ct1) mbar_wait(&bars[(k + 1) & 1], (unsigned)(((k + 1) >> 1) & 1), status);
      break;
    }
    const CT *sW = sWb + (size_t)(k & 1) * nm * EW_FC;
    const int4 *scol = scolb + (k & 1) * EW_FC;
    const int Mt = scol[0].w + 1;
    CT z[RA][4], z2[RA][4];
#pragma unroll
    for (int r = 0; r < RA; r++)
#pragma unroll
      for (int i = 0; i < 4; i++) {
        z[r][i] = cmk<T>((T)0, (T)0);
        z2[r][i] = cmk<T>((T)0, (T)0);
      }
    for (int m = 0; m < Mt; m++) {
      CT y[RA], ym[RA], w[4];
      const T fm = (T)m;
#pragma unroll
      for (int r = 0; r < RA; r++) {
        y[r] = sY[m * NA + ta + 16 * r];
        ym[r] = cmk<T>(fm * y[r].x, fm * y[r].y);
      }
#pragma unroll
      for (int i = 0; i < 4; i++) w[i] = sW[m * EW_FC + tc * 4 + i];
#pragma unroll
      for (int r = 0; r < RA; r++)
#pragma unroll
        for (int i = 0; i < 4; i++) {
          if (std::is_same<T, float>::value) {
            cmac(z[r][i], y[r], w[i]);
            cmac(z2[r][i], ym[r], w[i]);
          } else {
            // FP64: one product, reused (the FP64 pipe is the scarce one)
            const T pr = y[r].x * w[i].x - y[r].y * w[i].y;
            const T pi = y[r].x * w[i].y + y[r].y * w[i].x;
            z[r][i].x += pr;
            z[r][i].y += pi;
            z2[r][i].x += fm * pr;
            z2[r][i].y += fm * pi;
          }
        }
    }
    // epilogue: P = E0 E1 of each (atom, column), from the staged rows
#pragma unroll
    for (int i = 0; i < 4; i++) {
      const int4 col = scol[tc * 4 + i];
      if (col.z < 0) continue;
      const int ag0 = col.x < 0 ? -col.x : col.x, ag1 = col.y < 0 ? -col.y : col.y;
#pragma unroll
      for (int r = 0; r < RA; r++) {
        const CT *row = sE + (size_t)(ta + 16 * r) * LEs;
        CT e0 = row[ag0], e1 = row[G0 + 1 + ag1];
        if (col.x < 0) e0.y = -e0.y;
        if (col.y < 0) e1.y = -e1.y;
        const T pr = e0.x * e1.x - e0.y * e1.y;
        const T pi = e0.x * e1.y + e0.y * e1.x;
        const T im1 = pr * z[r][i].y + pi * z[r][i].x;
        const T im2 = pr * z2[r][i].y + pi * z2[r][i].x;
        acc[r][0].add((T)col.x * im1);
        acc[r][1].add((T)col.y * im1);
        acc[r][2].add(im2);
      }
    }
    __syncthreads();  // the buffer is refilled two tiles later
  }
  // reduce the 16 column groups of every atom in a fixed order
  __syncthreads();
  double *red = reinterpret_cast<double *>(smem_raw);  // [16][NA][3]
#pragma unroll
  for (int r = 0; r < RA; r++)
#pragma unroll
    for (int q = 0; q < 3; q++) red[((size_t)tc * NA + ta + 16 * r) * 3 + q] = acc[r][q].value();
  __syncthreads();
  double *out = part < 0 ? nullptr : piece + ((int64_t)(atile - nfull) * nsplit + part) * NA * 3;
  for (int v = threadIdx.x; v < NA * 3; v += blockDim.x) {
    const int la = v / 3, q = v % 3;
    const int a = abase + la;
    if (a >= a1) continue;
    double s = 0.0;
    for (int g = 0; g < 16; g++) s += red[((size_t)g * NA + la) * 3 + q];
    if (out) out[v] = s;
    else gfrac[(int64_t)a * 3 + q] = s;
  }
}

// Gradient sums of the split atom tiles: their pieces added in part order.
__global__ void k_ewald_force_combine(const double *__restrict__ piece, int a0, int a1, int NA, int nfull,
                                      int nsplit, double *__restrict__ gfrac) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t first = (int64_t)a0 + (int64_t)nfull * NA;
  if (idx >= (a1 - first) * 3) return;
  const int64_t la_all = idx / 3;
  const int q = (int)(idx % 3);
  const int64_t tile = la_all / NA;
  const int la = (int)(la_all % NA);
  double s = 0.0;
  for (int p = 0; p < nsplit; p++) s += piece[((tile * nsplit + p) * NA + la) * 3 + q];
  gfrac[(first + la_all) * 3 + q] = s;
}

// gpos = -2 pi (b0 f0 + b1 f1 + b2 f2) / dielectric (orig order).
__global__ void k_ewald_gpos(const double *__restrict__ gfrac, int64_t natom, CellGeom cell, double scale,
                             double *__restrict__ gpos) {
  int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (a >= natom) return;
  double f0 = gfrac[3 * a], f1 = gfrac[3 * a + 1], f2 = gfrac[3 * a + 2];
  for (int x = 0; x < 3; x++)
    gpos[3 * a + x] = scale * (f0 * cell.gv[x] + f1 * cell.gv[3 + x] + f2 * cell.gv[6 + x]);
}

__global__ void k_store_ewald_ev(const double *__restrict__ sums, double scale, double *__restrict__ ev) {
  if (threadIdx.x != 0) return;
  double e = sums[0];
  // vtens -= E on the diagonal, then the dielectric factor
  double v[9] = {sums[1] - e, sums[4], sums[5], sums[4], sums[2] - e, sums[6], sums[5], sums[6], sums[3] - e};
  ev[0] = e * scale;
  for (int q = 0; q < 9; q++) ev[1 + q] = v[q] * scale;
}

// Excluded-pair part of the Ewald correction (yaff/pes/ewald.c:290-335):
// one thread per scaling row, FP64, minimum image as in the reference.
__global__ void k_ewald_corr(const double *__restrict__ pos, const double *__restrict__ q, const int2 *__restrict__ ab,
                             const double *__restrict__ scale, int64_t n, CellGeom cell, double alpha, int64_t nlow,
                             int64_t nhigh, double inv_diel, double *__restrict__ gpos, double *__restrict__ partial) {
  __shared__ double red[8][7];
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double e = 0.0, v[6] = {0, 0, 0, 0, 0, 0};
  if (r < n) {
    int a = ab[r].x, b = ab[r].y;
    bool skip = (a < nlow && b < nlow) || (a >= nhigh && b >= nhigh);
    if (!skip) {
      double d[3] = {pos[3 * b] - pos[3 * a], pos[3 * b + 1] - pos[3 * a + 1], pos[3 * b + 2] - pos[3 * a + 2]};
      int m[3];
      exact_mic(d, cell, m);
      double dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      double x = alpha * dist;
      double pot = erf(x) / dist;
      double fac = (1.0 - scale[r]) * q[b] * q[a];
      double g = -fac * (1.1283791670955125739 * alpha * exp(-x * x) - pot) / dist / dist;
      e = -fac * pot * inv_diel;
      if (gpos) {
        for (int k = 0; k < 3; k++) {
          double y = d[k] * g * inv_diel;
          atomicAdd(gpos + 3 * b + k, y);
          atomicAdd(gpos + 3 * a + k, -y);
        }
      }
      g *= inv_diel;
      v[0] = d[0] * d[0] * g;
      v[1] = d[1] * d[1] * g;
      v[2] = d[2] * d[2] * g;
      v[3] = d[1] * d[0] * g;
      v[4] = d[2] * d[0] * g;
      v[5] = d[2] * d[1] * g;
    }
  }
  double vals[7] = {e, v[0], v[1], v[2], v[3], v[4], v[5]};
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 7; k++) {
    double x = vals[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    vals[k] = x;
  }
  if (lane == 0)
    for (int k = 0; k < 7; k++) red[wid][k] = vals[k];
  __syncthreads();
  if (threadIdx.x < 7) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w][threadIdx.x];
    partial[(int64_t)blockIdx.x * 7 + threadIdx.x] = s;
  }
}

__global__ void k_store_corr_ev(const double *__restrict__ sums, double eself, double *__restrict__ ev) {
  if (threadIdx.x != 0) return;
  ev[0] = sums[0] + eself;
  double v[9] = {sums[1], sums[4], sums[5], sums[4], sums[2], sums[6], sums[5], sums[6], sums[3]};
  for (int q = 0; q < 9; q++) ev[1 + q] = v[q];
}

// The bounded mbarrier wait of the kernels above on a barrier that nothing
// arrives at (no copy in flight): after `polls` polls the wait gives up and
// records YG_ST_TIMEOUT, exactly as a copy that never lands would make it.
__global__ void k_check_wait_timeout(int64_t polls, int *__restrict__ status) {
  __shared__ unsigned long long bar;
  if (threadIdx.x == 0) {
    mbar_init(&bar, 1);
    mbar_init_fence();
  }
  __syncwarp();
  if (threadIdx.x == 0) {
    bool done = false;
    for (int64_t it = 0; it < polls && !done; it++) {
      unsigned ok;
      asm volatile(
          "{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], 0;\nselp.u32 %0, 1, 0, p;\n}"
          : "=r"(ok)
          : "r"(smem_u32(&bar))
          : "memory");
      done = ok != 0;
    }
    if (!done) atomicOr(status + YG_ST_TIMEOUT, 1);
  }
}

}  // namespace

int yg_launch_check_wait_timeout(yg_ctx *ctx, int64_t polls) {
  k_check_wait_timeout<<<1, 32, 0, ctx->stream>>>(polls, ctx->d_status);
  YG_LAUNCH_CHECK(ctx, "k_check_wait_timeout");
  return YG_OK;
}

// Raises a kernel's dynamic shared-memory limit to the device's opt-in
// maximum, once per (kernel, device): setting it per launch to the launch's
// own size would race between host threads that drive different contexts.
int yg_smem_optin(const void *kernel, size_t need) {
  static std::mutex mu;
  static std::set<std::pair<const void *, int>> done;
  int dev = 0;
  YG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(mu);
  if (done.count(std::make_pair(kernel, dev))) return YG_OK;
  int optin = 0;
  YG_CUDA(cudaDeviceGetAttribute(&optin, cudaDevAttrMaxSharedMemoryPerBlockOptin, dev));
  cudaFuncAttributes fa;
  YG_CUDA(cudaFuncGetAttributes(&fa, kernel));
  optin -= (int)fa.sharedSizeBytes;  // static shared memory counts against the same limit
  if (need > (size_t)optin) {
    yg_set_error("Ewald tile needs more shared memory than the device offers");
    return YG_ERR_UNSUPPORTED;
  }
  YG_CUDA(cudaFuncSetAttribute(kernel, cudaFuncAttributeMaxDynamicSharedMemorySize, optin));
  done.insert(std::make_pair(kernel, dev));
  return YG_OK;
}

namespace {

// ---------------------------------------------------------------------------
// Tensor-core form of the mixed-precision reciprocal sum (G2 + 1 <= 32).
//
// Both passes are complex matrix products (S = X^T Y over atoms, Z = Y U
// over m), run here as warp-level FP16 MMAs (m16n8k16, FP32 accumulation).
// Every operand is split into FP16 hi + lo parts and a product is formed as
// hi*hi + hi*lo + lo*hi, which keeps about 22 significant bits; each
// 16-atom step of the S pass starts from a zero accumulator and is added to
// the running FP32 sums with round-to-nearest, so no error builds up inside
// the MMA accumulators.  Operands are scaled by powers of two into FP16
// range (charges by qscale, weights by s1 and, for the m-weighted product,
// s2) and unscaled exactly afterwards.
//
// Fragment layouts (m16n8k16; lane = 4 g + t):
//   A (16 x 16): a0 = A[g][2t..2t+1], a1 = A[g+8][2t..], a2 = A[g][2t+8..],
//                a3 = A[g+8][2t+8..];   B (16 x 8): b0 = B[2t..2t+1][g],
//                b1 = B[2t+8..2t+9][g];  D: d0,d1 = D[g][2t..], d2,d3 = D[g+8][2t..]
// with the lower column (row for B) in the low half of each register.

#define EW_MMA_KS 32   // atoms per S-pass stage (two 16-atom steps)
#ifndef EW_MMA_ATB
#define EW_MMA_ATB 512 // fewest atoms per S-pass block (the launch picks the chunk, a multiple of 32)
#endif
#ifndef YG_SFAC_PAIRS
#define YG_SFAC_PAIRS 1  // warp-MMA S pass over conjugate column pairs (X formed once per pair)
#endif
#ifndef EW_MMA_FT
#define EW_MMA_FT 4    // 4-column tiles per force-pass stage
#endif
#define EW_MMA_MAXR 8  // largest number of force-pass column ranges
#define EW_MMA_TEPAD 128  // zero E0|E1 rows past the last atom

__device__ __forceinline__ unsigned h2_bits(__half2 h) { return *reinterpret_cast<unsigned *>(&h); }

// (a, b) -> FP16 pairs hi = rn(a, b), lo = rn(a - hi, b - hi).
__device__ __forceinline__ void split_h2(float a, float b, unsigned &hi, unsigned &lo) {
  const __half2 h = __floats2half2_rn(a, b);
  const float2 f = __half22float2(h);
  hi = h2_bits(h);
  lo = h2_bits(__floats2half2_rn(a - f.x, b - f.y));
}

__device__ __forceinline__ void mma_f16(float (&d)[4], const unsigned (&a)[4], unsigned b0, unsigned b1) {
  asm("mma.sync.aligned.m16n8k16.row.col.f32.f16.f16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
      "{%0,%1,%2,%3};"
      : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
      : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// d = ah*bh + ah*bl + al*bh (d starts at zero).
__device__ __forceinline__ void mma_split(float (&d)[4], const unsigned (&ah)[4], const unsigned (&al)[4],
                                          unsigned bh0, unsigned bh1, unsigned bl0, unsigned bl1) {
  d[0] = d[1] = d[2] = d[3] = 0.f;
  mma_f16(d, ah, bh0, bh1);
  mma_f16(d, ah, bl0, bl1);
  mma_f16(d, al, bh0, bh1);
}

// MMA tables, 32 atoms per block of 256 threads: threads 0-95 form the
// fractional coordinate of one (atom, axis) each in FP64 and threads 96-127
// the scaled charges (FP64 work once per atom and axis, not once per atom
// and warp: the FP64 pipe is narrow); each warp then fills the rows of four
// atoms, its lanes taking one table entry each:
//   te[a][0..G0] = E0, te[a][G0+1..G0+G1+1] = E1 (float2, row stride lep);
//   yf[a][m] = (hi, lo) FP16 pairs of qscale q E2[m] (re in the low half),
//              m < nmf (zero beyond G2).
// The phases follow k_tables' FP32 form.
__global__ void __launch_bounds__(256) k_tables_mma(const double *__restrict__ pos, const double *__restrict__ charge,
                                                    int64_t natom, CellGeom cell, int G0, int G1, int G2,
                                                    float qscale, int lep, int nmf, float2 *__restrict__ te,
                                                    uint2 *__restrict__ yf) {
  __shared__ float s_sh[32][3], s_sl[32][3], s_q[32];
  const int t = threadIdx.x;
  const int64_t a0 = (int64_t)blockIdx.x * 32;
  if (t < 96) {
    const int la = t / 3, ax = t - 3 * (t / 3);
    const int64_t a = a0 + la;
    float sh = 0.f, sl = 0.f;
    if (a < natom) {
      const double *gv = cell.gv + 3 * ax;
      double sd = gv[0] * pos[3 * a] + gv[1] * pos[3 * a + 1] + gv[2] * pos[3 * a + 2];
      sd -= floor(sd);
      sh = (float)sd;
      sl = (float)(sd - (double)sh);
    }
    s_sh[la][ax] = sh;
    s_sl[la][ax] = sl;
  } else if (t < 128) {
    const int64_t a = a0 + (t - 96);
    s_q[t - 96] = a < natom ? (float)(charge[a] * (double)qscale) : 0.f;
  }
  __syncthreads();
  const int w = t >> 5, lane = t & 31;
  const int ne = G0 + G1 + 2;
  for (int k = 0; k < 4; k++) {
    const int la = 4 * w + k;
    const int64_t a = a0 + la;
    if (a >= natom) break;
    const float q = s_q[la];
    for (int slot = lane; slot < ne + nmf; slot += 32) {
      int g, ax;
      if (slot <= G0) {
        g = slot;
        ax = 0;
      } else if (slot < ne) {
        g = slot - (G0 + 1);
        ax = 1;
      } else {
        g = slot - ne;
        ax = 2;
      }
      const float s_hi = s_sh[la][ax], s_lo = s_sl[la][ax];
      const float fg = (float)g;
      const float pp = fg * s_hi;
      const float e = fmaf(fg, s_hi, -pp);
      const float x = (pp - rintf(pp)) + fmaf(fg, s_lo, e);
      float sn, c;
      sincospif(2.0f * x, &sn, &c);
      if (slot < ne) {
        te[a * lep + slot] = make_float2(c, sn);
      } else {
        const bool used = g <= G2;
        unsigned hi, lo;
        split_h2(used ? q * c : 0.f, used ? q * sn : 0.f, hi, lo);
        yf[a * nmf + g] = make_uint2(hi, lo);
      }
    }
  }
}

// The S pass's B fragments from yf: one thread per 16-byte unit (16-atom
// block, m < nms, component q (re, im), t < 4) =
// (hi(2t,2t+1), hi(2t+8,2t+9), lo(2t,2t+1), lo(2t+8,2t+9)).  Block positions
// are relative to the atom group ([lo, hi) first, then [0, lo), then [hi, N),
// each padded to a multiple of 16 atoms: bases 0, base1, base2), so a
// group's blocks hold only its own atoms; padding entries are zero.
__global__ void k_ys_mma(const uint2 *__restrict__ yf, int64_t natom, int64_t lo, int64_t hi, int64_t base1,
                         int64_t base2, int64_t nblocks, int nmf, int nms, uint4 *__restrict__ ys) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= nblocks * nms * 8) return;
  const int t = (int)(u & 3);
  const int comp = (int)((u >> 2) & 1);
  const int m = (int)((u >> 3) % nms);
  const int64_t blk = (u >> 3) / nms;
  const int64_t p0 = blk * 16;
  int64_t a0, n, gbase;
  if (p0 < base1) {
    a0 = lo; n = hi - lo; gbase = 0;
  } else if (p0 < base2) {
    a0 = 0; n = lo; gbase = base1;
  } else {
    a0 = hi; n = natom - hi; gbase = base2;
  }
  unsigned w[4] = {0u, 0u, 0u, 0u};
  const int ia[4] = {2 * t, 2 * t + 1, 2 * t + 8, 2 * t + 9};
  unsigned short hv[4], lv[4];
#pragma unroll
  for (int k = 0; k < 4; k++) {
    const int64_t r = p0 + ia[k] - gbase;
    hv[k] = 0;
    lv[k] = 0;
    if (r >= 0 && r < n && m < nmf) {
      const uint2 v = yf[(a0 + r) * nmf + m];
      hv[k] = (unsigned short)(comp == 0 ? (v.x & 0xffffu) : (v.x >> 16));
      lv[k] = (unsigned short)(comp == 0 ? (v.y & 0xffffu) : (v.y >> 16));
    }
  }
  w[0] = (unsigned)hv[0] | ((unsigned)hv[1] << 16);
  w[1] = (unsigned)hv[2] | ((unsigned)hv[3] << 16);
  w[2] = (unsigned)lv[0] | ((unsigned)lv[1] << 16);
  w[3] = (unsigned)lv[2] | ((unsigned)lv[3] << 16);
  ys[u] = make_uint4(w[0], w[1], w[2], w[3]);
}

// S pass on the tensor cores.  grid = (atom chunks of atb atoms, 64-column
// tiles, m slabs); 4 warps, warp w owns columns 16 w .. 16 w + 15 of the
// tile as two 8-column MMA row tiles (rows 0-7: Re X, rows 8-15: Im X) and
// NT n-tiles of 4 m values (columns 0-3: Re Y, 4-7: Im Y) of the slab.  The
// E0|E1 rows and the Y fragments of 32 atoms at a time arrive by
// double-buffered bulk copies (te holds 32 rows past the last atom, ys two
// blocks past the last group).  Partial layout as k_sfac with 64 columns
// ([chunk][tile][slab][c][m]), or with 128 over conjugate pairs (PR below:
// a tile of 64 pairs, the warps own 16 pairs each).
template <int NT>
__device__ __forceinline__ void sfac_mma_stage(const float2 *__restrict__ sTE, const uint4 *__restrict__ sYS, int lep,
                                               int nms, int mb, int nrow, const int (&o0)[2], const int (&o1)[2],
                                               const float (&sg0)[2], const float (&sg1)[2], const float (&ok)[2],
                                               int g, int t, float (&acc)[2][8][4]) {
#pragma unroll 1
  for (int kk = 0; kk < 2; kk++) {
    if (kk * 16 >= nrow) break;
    unsigned ah[2][4], al[2][4];
#pragma unroll
    for (int j = 0; j < 2; j++) {
      float xr[4], xi[4];
#pragma unroll
      for (int u = 0; u < 4; u++) {
        const int la = kk * 16 + 2 * t + (u & 1) + (u >> 1) * 8;  // atoms 2t, 2t+1, 2t+8, 2t+9
        const float2 *row = sTE + (size_t)la * lep;
        float2 e0 = row[o0[j]], e1 = row[o1[j]];
        e0.x *= ok[j];
        e0.y *= sg0[j] * ok[j];
        e1.y *= sg1[j];
        xr[u] = e0.x * e1.x - e0.y * e1.y;
        xi[u] = e0.x * e1.y + e0.y * e1.x;
      }
      split_h2(xr[0], xr[1], ah[j][0], al[j][0]);
      split_h2(xi[0], xi[1], ah[j][1], al[j][1]);
      split_h2(xr[2], xr[3], ah[j][2], al[j][2]);
      split_h2(xi[2], xi[3], ah[j][3], al[j][3]);
    }
#pragma unroll
    for (int nt = 0; nt < NT; nt++) {
      const uint4 b = sYS[(((size_t)kk * nms + mb + nt * 4 + (g & 3)) * 2 + (g >> 2)) * 4 + t];
#pragma unroll
      for (int j = 0; j < 2; j++) {
        float d[4];
        mma_split(d, ah[j], al[j], b.x, b.y, b.z, b.w);
#pragma unroll
        for (int e = 0; e < 4; e++) acc[j][nt][e] += d[e];
      }
    }
  }
}

// PR (conjugate pairs): cols is the pair list, 128 slots per tile (64 '+'
// members, then their partners); X is formed for the '+' members only and
// each accumulator gives both columns: S(g0, g1) = (RR - II, RI + IR) and
// S(-g0, -g1) = (RR + II, RI - IR) from the sums RR = Re X Re Y, II = Im X Im
// Y, RI = Re X Im Y, IR = Im X Re Y.
template <bool PR>
__global__ void __launch_bounds__(128) k_sfac_mma(const float2 *__restrict__ te, const uint4 *__restrict__ ys,
                                                  int n, int G0, int lep, int nms,
                                                  const int4 *__restrict__ cols, float2 *__restrict__ Spart,
                                                  int ntile, int nslab, int atb, int *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_mma[];
  __shared__ unsigned long long bars[2];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int tile = blockIdx.y, slab = blockIdx.z;
  const int mb = slab * EW_MS;
  const size_t te_bytes = (size_t)EW_MMA_KS * lep * sizeof(float2);
  const size_t ys_bytes = (size_t)(EW_MMA_KS / 16) * nms * 2 * 4 * sizeof(uint4);
  const size_t stage = te_bytes + ys_bytes;
  constexpr int SC = PR ? 128 : 64;      // partial columns per tile
  const int wc0 = tile * SC + w * 16;  // the warp's first column (largest extent)
  const int Mw = cols[wc0].w + 1 - mb;
  const int nt = Mw > 0 ? min(8, (Mw + 3) / 4) : 0;
  int o0[2], o1[2];
  float sg0[2], sg1[2], ok[2];
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const int4 col = cols[wc0 + 8 * j + g];
    o0[j] = col.x < 0 ? -col.x : col.x;
    o1[j] = G0 + 1 + (col.y < 0 ? -col.y : col.y);
    sg0[j] = col.x < 0 ? -1.f : 1.f;
    sg1[j] = col.y < 0 ? -1.f : 1.f;
    ok[j] = col.z >= 0 ? 1.f : 0.f;
  }
  float acc[2][8][4];
#pragma unroll
  for (int j = 0; j < 2; j++)
#pragma unroll
    for (int n = 0; n < 8; n++)
#pragma unroll
      for (int e = 0; e < 4; e++) acc[j][n][e] = 0.f;
  // te, ys start at the group's first atom and first 16-atom block
  const int abeg = blockIdx.x * atb;
  const int aend = min(n, abeg + atb);
  const int tmax = cols[tile * SC].w + 1 - mb;    // the block's largest extent
  if (tmax > 0 && aend > abeg) {
    const int nstage = (aend - abeg + EW_MMA_KS - 1) / EW_MMA_KS;
    if (threadIdx.x == 0) {
      mbar_init(&bars[0], 1);
      mbar_init(&bars[1], 1);
      mbar_init_fence();
    }
    __syncthreads();
    // stage s: the 32 padded rows from abeg + 32 s (te, ys of two 16-atom blocks)
    auto issue = [&](int s) {
      const int ab = abeg + s * EW_MMA_KS;
      unsigned char *dst = smem_mma + (size_t)(s & 1) * stage;
      unsigned long long *bar = &bars[s & 1];
      bulk_expect(bar, (unsigned)stage);
      bulk_copy(dst, te + (size_t)ab * lep, (unsigned)te_bytes, bar);
      bulk_copy(dst + te_bytes, ys + (size_t)(ab / 16) * nms * 2 * 4, (unsigned)ys_bytes, bar);
    };
    if (threadIdx.x == 0) issue(0);
    for (int s = 0; s < nstage; s++) {
      if (threadIdx.x == 0 && s + 1 < nstage) issue(s + 1);
      const bool arrived = mbar_wait(&bars[s & 1], (unsigned)((s >> 1) & 1), status);
      if (__syncthreads_or(!arrived)) {
        if (threadIdx.x == 0 && s + 1 < nstage) mbar_wait(&bars[(s + 1) & 1], (unsigned)(((s + 1) >> 1) & 1), status);
        break;
      }
      const unsigned char *buf = smem_mma + (size_t)(s & 1) * stage;
      const float2 *sTE = reinterpret_cast<const float2 *>(buf);
      const uint4 *sYS = reinterpret_cast<const uint4 *>(buf + te_bytes);
      const int nrow = min(EW_MMA_KS, aend - (abeg + s * EW_MMA_KS));
      switch (nt) {
        case 8: sfac_mma_stage<8>(sTE, sYS, lep, nms, mb, nrow, o0, o1, sg0, sg1, ok, g, t, acc); break;
        case 7: sfac_mma_stage<7>(sTE, sYS, lep, nms, mb, nrow, o0, o1, sg0, sg1, ok, g, t, acc); break;
        case 6: sfac_mma_stage<6>(sTE, sYS, lep, nms, mb, nrow, o0, o1, sg0, sg1, ok, g, t, acc); break;
        case 5: sfac_mma_stage<5>(sTE, sYS, lep, nms, mb, nrow, o0, o1, sg0, sg1, ok, g, t, acc); break;
        case 4: sfac_mma_stage<4>(sTE, sYS, lep, nms, mb, nrow, o0, o1, sg0, sg1, ok, g, t, acc); break;
        case 3: sfac_mma_stage<3>(sTE, sYS, lep, nms, mb, nrow, o0, o1, sg0, sg1, ok, g, t, acc); break;
        case 2: sfac_mma_stage<2>(sTE, sYS, lep, nms, mb, nrow, o0, o1, sg0, sg1, ok, g, t, acc); break;
        case 1: sfac_mma_stage<1>(sTE, sYS, lep, nms, mb, nrow, o0, o1, sg0, sg1, ok, g, t, acc); break;
        default: break;
      }
      __syncthreads();  // the buffer is refilled two stages later
    }
  }
  // S = (Re X Re Y - Im X Im Y) + i (Re X Im Y + Im X Re Y): lanes t and t^2
  // hold the Re Y and Im Y columns of the same two m values
  const int64_t base = (((int64_t)blockIdx.x * ntile + tile) * nslab + slab) * (SC * EW_MS);
#pragma unroll
  for (int j = 0; j < 2; j++) {
    const int c = w * 16 + 8 * j + g;
#pragma unroll
    for (int n = 0; n < 8; n++) {
      const float p2 = __shfl_xor_sync(0xffffffffu, acc[j][n][2], 2);
      const float p3 = __shfl_xor_sync(0xffffffffu, acc[j][n][3], 2);
      if (n >= nt) continue;
      const int m = n * 4 + 2 * (t & 1);
      float *dst = reinterpret_cast<float *>(Spart + base + (int64_t)c * EW_MS + m);
      float *dcj = reinterpret_cast<float *>(Spart + base + (int64_t)(64 + c) * EW_MS + m);
      if (t < 2) {
        dst[0] = acc[j][n][0] - p2;  // Re S(m), Re S(m + 1)
        dst[2] = acc[j][n][1] - p3;
        if (PR) {
          dcj[0] = acc[j][n][0] + p2;  // the partner's Re S(m), Re S(m + 1)
          dcj[2] = acc[j][n][1] + p3;
        }
      } else {
        dst[1] = acc[j][n][0] + p2;  // Im S(m), Im S(m + 1)
        dst[3] = acc[j][n][1] + p3;
        if (PR) {
          dcj[1] = acc[j][n][0] - p2;  // the partner's Im S(m), Im S(m + 1)
          dcj[3] = acc[j][n][1] - p3;
        }
      }
    }
  }
}

// Force pass on the tensor cores.  grid = (blocks of 128 atoms, column
// ranges); one warp per 16 atoms, 8 warps per block; every warp sweeps the
// 4-column tiles [crange[r], crange[r+1]) of its range r.  Z = sum_m Y U and
// Z2 = sum_m m Y U (U = the stored conj weights) come from MMAs with
// M = 16 atoms, N = 4 columns x (re, im), K = 8 m x (re, im) per step; the Y
// fragments of the warp's atoms stay in registers, the block's E0|E1 rows
// are staged in shared memory once, and the weight fragments of EW_MMA_FT
// tiles at a time arrive by double-buffered bulk copies.  A weight unit
// (1 KB per tile and 8 m values) holds the Z fragments of the 32 lanes
// (16 B each) and then the Z2 fragments, so each fragment load reads 512
// contiguous bytes.  The epilogue forms P = E0 E1 per (atom, column) and
// accumulates g0 Im(P Z), g1 Im(P Z), Im(P Z2).  With one range the sums go
// to gfrac; with several to out[r][atom][3] for k_ewald_force_mma_combine.
#ifndef YG_FM_MINB
#define YG_FM_MINB 2  // resident tensor-core force-pass blocks per SM the register budget is sized for
#endif
__global__ void __launch_bounds__(256, YG_FM_MINB) k_ewald_force_mma(const float2 *__restrict__ te, const uint2 *__restrict__ yf,
                                                         int a0, int a1, int G0, int lep, int nmf, int nks,
                                                         const int4 *__restrict__ cols, const int *__restrict__ crange,
                                                         const int *__restrict__ woff, const uint4 *__restrict__ wb,
                                                         double inv1, double inv2, double *__restrict__ out,
                                                         int64_t rstride, int *__restrict__ status) {
  extern __shared__ __align__(16) unsigned char smem_mma[];
  __shared__ unsigned long long bars[3];
  const int lane = threadIdx.x & 31, w = threadIdx.x >> 5;
  const int g = lane >> 2, t = lane & 3;
  const int bbase = a0 + blockIdx.x * 128;
  const int wbase = bbase + w * 16;
  const int cr0 = crange[blockIdx.y], cr1 = crange[blockIdx.y + 1];
  const size_t te_bytes = (size_t)128 * lep * sizeof(float2);
  const int stage_units = EW_MMA_FT * nks;  // 1 KB units per stage (max)
  const size_t stage = (size_t)stage_units * 1024 + EW_MMA_FT * 4 * sizeof(int4);
  const float2 *sTE = reinterpret_cast<const float2 *>(smem_mma);
  unsigned char *sbuf = smem_mma + te_bytes;
  if (threadIdx.x == 0) {
    mbar_init(&bars[0], 1);
    mbar_init(&bars[1], 1);
    mbar_init(&bars[2], 1);
    mbar_init_fence();
  }
  __syncthreads();
  // the block's 128 E0|E1 rows (te holds 128 zero rows past the last atom)
  if (threadIdx.x == 0) bulk_load(smem_mma, te + (size_t)bbase * lep, (unsigned)te_bytes, &bars[2]);
  // Y fragments of the warp's atoms (atoms past the group read zeros)
  unsigned yh[4][4], yl[4][4];
  const int ra = min(wbase + g, a1 - 1), rb = min(wbase + g + 8, a1 - 1);
  const bool va = wbase + g < a1, vb = wbase + g + 8 < a1;
#pragma unroll
  for (int ks = 0; ks < 4; ks++) {
    if (ks < nks) {
      const int m0 = ks * 8 + t, m1 = m0 + 4;
      uint2 v;
      v = yf[(size_t)ra * nmf + m0]; yh[ks][0] = va ? v.x : 0u; yl[ks][0] = va ? v.y : 0u;
      v = yf[(size_t)rb * nmf + m0]; yh[ks][1] = vb ? v.x : 0u; yl[ks][1] = vb ? v.y : 0u;
      v = yf[(size_t)ra * nmf + m1]; yh[ks][2] = va ? v.x : 0u; yl[ks][2] = va ? v.y : 0u;
      v = yf[(size_t)rb * nmf + m1]; yh[ks][3] = vb ? v.x : 0u; yl[ks][3] = vb ? v.y : 0u;
    } else {
#pragma unroll
      for (int e = 0; e < 4; e++) yh[ks][e] = yl[ks][e] = 0u;
    }
  }
  const float2 *rowa = sTE + (size_t)(w * 16 + g) * lep, *rowb = rowa + (size_t)8 * lep;
  CompAcc<float> acc[2][3];
#pragma unroll
  for (int r = 0; r < 2; r++)
#pragma unroll
    for (int q = 0; q < 3; q++) acc[r][q].init();
  const int nstage = (cr1 - cr0 + EW_MMA_FT - 1) / EW_MMA_FT;
  auto issue = [&](int s) {
    const int t0 = cr0 + s * EW_MMA_FT, t1 = min(cr1, t0 + EW_MMA_FT);
    unsigned char *dst = sbuf + (size_t)(s & 1) * stage;
    const unsigned wbytes = (unsigned)(woff[t1] - woff[t0]) * 1024u;
    const unsigned cbytes = (unsigned)((t1 - t0) * 4 * sizeof(int4));
    unsigned long long *bar = &bars[s & 1];
    bulk_expect(bar, wbytes + cbytes);
    bulk_copy(dst, wb + (size_t)woff[t0] * 64, wbytes, bar);
    bulk_copy(dst + (size_t)stage_units * 1024, cols + t0 * 4, cbytes, bar);
  };
  if (threadIdx.x == 0 && nstage > 0) issue(0);
  bool ok_te = mbar_wait(&bars[2], 0, status);
  if (__syncthreads_or(!ok_te)) {
    if (threadIdx.x == 0 && nstage > 0) mbar_wait(&bars[0], 0, status);
    return;
  }
  for (int s = 0; s < nstage; s++) {
    if (threadIdx.x == 0 && s + 1 < nstage) issue(s + 1);
    const bool arrived = mbar_wait(&bars[s & 1], (unsigned)((s >> 1) & 1), status);
    if (__syncthreads_or(!arrived)) {
      if (threadIdx.x == 0 && s + 1 < nstage) mbar_wait(&bars[(s + 1) & 1], (unsigned)(((s + 1) >> 1) & 1), status);
      break;
    }
    const unsigned char *buf = sbuf + (size_t)(s & 1) * stage;
    const uint4 *fr = reinterpret_cast<const uint4 *>(buf);
    const int4 *scol = reinterpret_cast<const int4 *>(buf + (size_t)stage_units * 1024);
    const int nt = min(cr1, cr0 + s * EW_MMA_FT + EW_MMA_FT) - (cr0 + s * EW_MMA_FT);
    float ps[2][3] = {{0.f, 0.f, 0.f}, {0.f, 0.f, 0.f}};
    // all MMAs of the stage's tiles first, then their epilogues: the FP32
    // epilogue of one tile overlaps the MMAs of the next still in flight
    float z[EW_MMA_FT][4], z2[EW_MMA_FT][4];
    int ku = 0;  // first unit of the tile in the stage
#pragma unroll
    for (int j = 0; j < EW_MMA_FT; j++) {
#pragma unroll
      for (int e = 0; e < 4; e++) z[j][e] = z2[j][e] = 0.f;
      if (j < nt) {
        const int kn = (scol[j * 4].w + 8) >> 3;  // the tile's k-steps: its first column's extent
#pragma unroll
        for (int ks = 0; ks < 4; ks++) {
          if (ks < kn) {
            const uint4 b1 = fr[(ku + ks) * 64 + lane], b2 = fr[(ku + ks) * 64 + 32 + lane];
            mma_f16(z[j], yh[ks], b1.x, b1.y);
            mma_f16(z[j], yh[ks], b1.z, b1.w);
            mma_f16(z[j], yl[ks], b1.x, b1.y);
            mma_f16(z2[j], yh[ks], b2.x, b2.y);
            mma_f16(z2[j], yh[ks], b2.z, b2.w);
            mma_f16(z2[j], yl[ks], b2.x, b2.y);
          }
        }
        ku += kn;
      }
    }
#pragma unroll
    for (int j = 0; j < EW_MMA_FT; j++) {
      if (j >= nt) break;
      // z[j][0], z[j][1]: Z of (atom g, column t); z[j][2], z[j][3]: atom g + 8
      const int4 col = scol[j * 4 + t];
      if (col.z >= 0) {
        const int ag0 = col.x < 0 ? -col.x : col.x, ag1 = G0 + 1 + (col.y < 0 ? -col.y : col.y);
        const float sx = col.x < 0 ? -1.f : 1.f, sy = col.y < 0 ? -1.f : 1.f;
#pragma unroll
        for (int r = 0; r < 2; r++) {
          const float2 *row = r ? rowb : rowa;
          const float2 e0 = row[ag0], e1 = row[ag1];
          const float e0y = sx * e0.y, e1y = sy * e1.y;
          const float pr = e0.x * e1.x - e0y * e1y;
          const float pi = e0.x * e1y + e0y * e1.x;
          const float im1 = pr * z[j][2 * r + 1] + pi * z[j][2 * r];
          const float im2 = pr * z2[j][2 * r + 1] + pi * z2[j][2 * r];
          ps[r][0] += (float)col.x * im1;
          ps[r][1] += (float)col.y * im1;
          ps[r][2] += im2;
        }
      }
    }
#pragma unroll
    for (int r = 0; r < 2; r++)
#pragma unroll
      for (int q = 0; q < 3; q++) acc[r][q].add(ps[r][q]);
    __syncthreads();  // the buffer is refilled two stages later
  }
  // sum the four column lanes of every atom (fixed order), unscale, store
  double *dst = out + (int64_t)blockIdx.y * rstride;
#pragma unroll
  for (int r = 0; r < 2; r++) {
    double v[3];
#pragma unroll
    for (int q = 0; q < 3; q++) {
      v[q] = acc[r][q].value();
      v[q] += __shfl_xor_sync(0xffffffffu, v[q], 1);
      v[q] += __shfl_xor_sync(0xffffffffu, v[q], 2);
    }
    const int a = wbase + g + 8 * r;
    if (t == 0 && a < a1) {
      dst[(int64_t)a * 3] = v[0] * inv1;
      dst[(int64_t)a * 3 + 1] = v[1] * inv1;
      dst[(int64_t)a * 3 + 2] = v[2] * inv2;
    }
  }
}

// gfrac of atoms [a0, a1) = the sum of the column ranges' parts, in order.
__global__ void k_ewald_force_mma_combine(const double *__restrict__ part, int64_t rstride, int nrange, int a0,
                                          int a1, double *__restrict__ gfrac) {
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= (int64_t)(a1 - a0) * 3) return;
  const int64_t k = (int64_t)a0 * 3 + idx;
  double s = 0.0;
  for (int r = 0; r < nrange; r++) s += part[r * rstride + k];
  gfrac[k] = s;
}

// Blocks of a kernel the device holds at once (all SMs), cached per
// (kernel, dynamic shared memory).
static int resident_blocks(const void *fn, int threads, size_t smem, yg_occ *oc, int *blocks) {
  if (oc->fn != fn || oc->smem != smem || oc->blocks <= 0) {
    int dev = 0, nsm = 0, occ = 0;
    YG_CUDA(cudaGetDevice(&dev));
    YG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    YG_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&occ, fn, threads, smem));
    if (occ < 1) {
      yg_set_error("Ewald kernel does not fit on a multiprocessor");
      return YG_ERR_UNSUPPORTED;
    }
    oc->fn = fn;
    oc->smem = smem;
    oc->blocks = occ * nsm;
  }
  *blocks = oc->blocks;
  return YG_OK;
}

template <typename T> size_t force_smem(int G0, int G1, int nm, int RA) {
  const size_t ct = sizeof(typename C2<T>::t);
  size_t a = (size_t)nm * 16 * RA * ct + (size_t)16 * RA * ((G0 + G1 + 2) | 1) * ct + (size_t)2 * nm * EW_FC * ct +
             2 * EW_FC * sizeof(int4);
  size_t b = (size_t)16 * 16 * RA * 3 * sizeof(double);
  return a > b ? a : b;
}

template <typename T, typename TA, int RA>
int run_reci(yg_ctx *ctx, int want_grad) {
  typedef typename C2<T>::t CT;
  typedef typename C2<TA>::t CA;
  const int G0 = (int)ctx->ew_gmax[0], G1 = (int)ctx->ew_gmax[1], G2 = (int)ctx->ew_gmax[2];
  const int nm = G2 + 1;
  const int64_t N = ctx->natom;
  const int nstile = ctx->ew_ntile;
  const int nftile = ctx->ew_nftile;              // force tiles with work
  const int64_t wstride = (int64_t)2 * nstile * nm * EW_FC;  // tiled weights per group
  const int nslab = (nm + EW_MS - 1) / EW_MS;
  const int ATB = SfacCfg<T>::ATB;
  const int64_t nk_dense = (int64_t)ctx->ew_ncol * nm;
  int rc;
  // tables
  const int Lp = ew_row_stride(G0, G1, G2);
  size_t tb = (size_t)N * Lp * sizeof(CT);
  if ((rc = yg_ensure(ctx, &ctx->d_ew_tab, &ctx->ew_bytes_tab, tb))) return rc;
  CT *tab = (CT *)ctx->d_ew_tab;
  k_tables<T><<<yg_blocks(N * 3, 128), 128, 0, ctx->stream>>>(ctx->d_pos, ctx->d_charge, N, ctx->cell, G0, G1, G2, tab);
  YG_LAUNCH_CHECK(ctx, "k_tables");
  // atom groups: 0 = [nlow, nhigh) (always), 1 = [0, nlow), 2 = [nhigh, N)
  int64_t lo = ctx->ew_nlow, hi = ctx->ew_nhigh;
  int64_t gb[3][2] = {{lo, hi}, {0, lo}, {hi, N}};
  const int nS = (lo > 0 || hi < N) ? 3 : 1;
  // structure factors
  int maxchunk = 0;
  for (int g = 0; g < nS; g++) {
    int64_t n = gb[g][1] - gb[g][0];
    int nch = (int)((n + ATB - 1) / ATB);
    if (nch > maxchunk) maxchunk = nch;
  }
  if (maxchunk < 1) maxchunk = 1;
  size_t per = (size_t)nstile * nslab * EW_SC * EW_MS;
  if ((rc = yg_ensure(ctx, &ctx->d_ew_Spart, &ctx->ew_bytes_Spart, per * maxchunk * sizeof(CA)))) return rc;
  for (int g = 0; g < nS; g++) {
    int64_t n = gb[g][1] - gb[g][0];
    double *S = ctx->d_ew_S + (size_t)g * 2 * nk_dense;
    if (n <= 0) {
      YG_CUDA(cudaMemsetAsync(S, 0, 2 * nk_dense * sizeof(double), ctx->stream));
      continue;
    }
    int nch = (int)((n + ATB - 1) / ATB);
    dim3 grid(nch, nstile, nslab);
    YG_CUDA(cudaMemsetAsync(S, 0, 2 * nk_dense * sizeof(double), ctx->stream));
    const size_t ssm = (size_t)2 * SfacCfg<T>::KA * Lp * sizeof(CT);
    if ((rc = yg_smem_optin((const void *)k_sfac<T, TA>, ssm))) return rc;
    k_sfac<T, TA><<<grid, 128, ssm, ctx->stream>>>(tab, (int)gb[g][0], (int)gb[g][1], G0, G1, G2,
                                                 (const int4 *)ctx->d_ew_tiles, (CA *)ctx->d_ew_Spart, nstile, nslab,
                                                 ctx->d_status);
    YG_LAUNCH_CHECK(ctx, "k_sfac");
    k_sfac_reduce<TA><<<yg_blocks((int64_t)per * 4, 256), 256, 0, ctx->stream>>>(
        (const CA *)ctx->d_ew_Spart, nch, nstile, nslab, EW_SC, (const int4 *)ctx->d_ew_tiles, nm, 1.0, S);
    YG_LAUNCH_CHECK(ctx, "k_sfac_reduce");
  }
  // energy, virial, weights
  const int ngroup = (nS == 3) ? 3 : 1;
  if ((rc = yg_ensure(ctx, &ctx->d_ew_W, &ctx->ew_bytes_W, (size_t)ngroup * wstride * sizeof(CT)))) return rc;
  // padding slots of the tiled weights stay zero
  YG_CUDA(cudaMemsetAsync(ctx->d_ew_W, 0, (size_t)ngroup * wstride * sizeof(CT), ctx->stream));
  const int eb = yg_blocks(nk_dense, 256);
  if ((rc = yg_ensure(ctx, (void **)&ctx->d_ew_red, &ctx->ew_red_cap, ((size_t)eb * 7 + 64 + 7) * sizeof(double))))
    return rc;
  double *partial = ctx->d_ew_red + 64;
  const double fac2 = 0.25 / ctx->ew_alpha / ctx->ew_alpha;
  k_ewald_energy<T><<<eb, 256, 0, ctx->stream>>>(ctx->d_ew_S, nS, nk_dense, ctx->d_ew_pref, G0, G1, nm, ctx->cell,
                                                fac2, ngroup, ctx->d_ew_wslot, wstride, (CT *)ctx->d_ew_W,
                                                nullptr, nullptr, 0, nullptr, nullptr, 0, nullptr, 0.0, 0.0, partial);
  YG_LAUNCH_CHECK(ctx, "k_ewald_energy");
  double *sums = partial + (size_t)eb * 7;
  if ((rc = yg_launch_reduce_ev(ctx, partial, eb, 7, sums))) return rc;
  double *ev = ctx->d_part_ev + 10 * YG_PART_EWALD_RECI;
  k_store_ewald_ev<<<1, 32, 0, ctx->stream>>>(sums, 1.0 / ctx->ew_diel, ev);
  YG_LAUNCH_CHECK(ctx, "k_store_ewald_ev");
  double *gpos = ctx->d_part_gpos + (size_t)YG_PART_EWALD_RECI * N * 3;
  if (!want_grad) {
    YG_CUDA(cudaMemsetAsync(gpos, 0, N * 3 * sizeof(double), ctx->stream));
    ctx->part_valid[YG_PART_EWALD_RECI] = 1;
    return YG_OK;
  }
  // force pass, per atom group
  if ((rc = yg_ensure(ctx, (void **)&ctx->d_ew_gpart, &ctx->ew_bytes_gpart, (size_t)N * 3 * sizeof(double)))) return rc;
  size_t smem = force_smem<T>(G0, G1, nm, RA);
  if ((rc = yg_smem_optin((const void *)k_ewald_force<T, RA>, smem))) return rc;
  const int NA = 16 * RA;
  int slots;
  if ((rc = resident_blocks((const void *)k_ewald_force<T, RA>, 256, smem, &ctx->ew_occ_f, &slots))) return rc;
  for (int g = 0; g < nS; g++) {
    int64_t n = gb[g][1] - gb[g][0];
    if (n <= 0) continue;
    const CT *Wg = (const CT *)ctx->d_ew_W + (size_t)(ngroup == 1 ? 0 : g) * wstride;
    // whole atom tiles fill the full waves; the tiles of the last, partial
    // wave are split over column ranges so that it is as full as the others
    const int nat = (int)((n + NA - 1) / NA);
    const int rem = nat % slots;
    int nsplit = rem > 0 ? std::min(nftile, slots / rem) : 1;
    if (nsplit < 2) nsplit = 1;
    const int nfull = nsplit > 1 ? nat - rem : nat;
    const int nblk = nfull + (nat - nfull) * nsplit;
    if (nsplit > 1) {
      const size_t pbytes = (size_t)(nat - nfull) * nsplit * NA * 3 * sizeof(double);
      if ((rc = yg_ensure(ctx, (void **)&ctx->d_ew_fpiece, &ctx->ew_bytes_fpiece, pbytes))) return rc;
    }
    k_ewald_force<T, RA><<<nblk, 256, smem, ctx->stream>>>(tab, (int)gb[g][0], (int)gb[g][1], G0, G1, G2,
                                                          (const int4 *)ctx->d_ew_tiles, nftile, ctx->d_ew_fpre,
                                                          nfull, nsplit, Wg, ctx->d_ew_gpart, ctx->d_ew_fpiece,
                                                          ctx->d_status);
    YG_LAUNCH_CHECK(ctx, "k_ewald_force");
    if (nsplit > 1) {
      k_ewald_force_combine<<<yg_blocks((n - (int64_t)nfull * NA) * 3, 256), 256, 0, ctx->stream>>>(
          ctx->d_ew_fpiece, (int)gb[g][0], (int)gb[g][1], NA, nfull, nsplit, ctx->d_ew_gpart);
      YG_LAUNCH_CHECK(ctx, "k_ewald_force_combine");
    }
  }
  k_ewald_gpos<<<yg_blocks(N, 256), 256, 0, ctx->stream>>>(ctx->d_ew_gpart, N, ctx->cell,
                                                           -6.2831853071795864769 / ctx->ew_diel, gpos);
  YG_LAUNCH_CHECK(ctx, "k_ewald_gpos");
  ctx->part_valid[YG_PART_EWALD_RECI] = 1;
  return YG_OK;
}


// Smallest power of two >= x (x > 0), as a double.
static double pow2_ceil(double x) { return std::ldexp(1.0, (int)std::ceil(std::log2(x))); }

// The mixed-precision reciprocal sum on the tensor cores (G2 + 1 <= 32).
int run_reci_mma(yg_ctx *ctx, int want_grad) {
  const int G0 = (int)ctx->ew_gmax[0], G1 = (int)ctx->ew_gmax[1], G2 = (int)ctx->ew_gmax[2];
  const int nm = G2 + 1;
  const int64_t N = ctx->natom;
  const int ntile64 = 2 * ctx->ew_ntile;
  const int64_t nk_dense = (int64_t)ctx->ew_ncol * nm;
  const int lep = (G0 + G1 + 2 + 1) & ~1;  // E0|E1 row, even: 16-byte rows
  const int nks = (nm + 7) / 8, nmf = 8 * nks, nms = (nm + 3) & ~3;
  int rc;
  // atom groups: 0 = [nlow, nhigh) (always), 1 = [0, nlow), 2 = [nhigh, N)
  const int64_t lo = ctx->ew_nlow, hi = ctx->ew_nhigh;
  const int64_t gb[3][2] = {{lo, hi}, {0, lo}, {hi, N}};
  const int nS = (lo > 0 || hi < N) ? 3 : 1;
  auto r16 = [](int64_t n) { return (n + 15) / 16 * 16; };
  const int64_t gbase[3] = {0, r16(hi - lo), r16(hi - lo) + r16(lo)};
  const int64_t ys_blocks = (r16(hi - lo) + r16(lo) + r16(N - hi)) / 16 + 2;
  // operand scales (powers of two): |qscale q| <= 1; |s1 U| <= 2^13 and
  // |s2 m U| <= 2^13 with |U| <= 2 max A sum |q|
  const double qmax = ctx->h_qmax, qsum = ctx->h_qsum;
  const double qscale = qmax > 0.0 ? 1.0 / pow2_ceil(qmax) : 1.0;
  const double ub = 2.0 * ctx->ew_amax * qsum;
  const double s1 = ub > 0.0 ? 8192.0 / pow2_ceil(ub) : 1.0;
  const double s2 = s1 / pow2_ceil(std::max(1, G2));
  // tables
  if ((rc = yg_ensure(ctx, &ctx->d_ew_te, &ctx->ew_bytes_te, (size_t)(N + EW_MMA_TEPAD) * lep * sizeof(float2))))
    return rc;
  if ((rc = yg_ensure(ctx, &ctx->d_ew_yf, &ctx->ew_bytes_yf, (size_t)N * nmf * sizeof(uint2)))) return rc;
  // S pass: the warp-level MMA form (faster here), or on request the tcgen05
  // form (B operand nks KB per 16-atom block) where its staging fits
  const bool usf = ctx->ew_sfac_path == 2 && nks <= yg_umma_kmax() && yg_umma_sfac_smem(lep) > 0;
  const size_t ys_bytes = usf ? (size_t)ys_blocks * nks * 1024 : (size_t)ys_blocks * nms * 8 * sizeof(uint4);
  if ((rc = yg_ensure(ctx, &ctx->d_ew_ys, &ctx->ew_bytes_ys, ys_bytes))) return rc;
  float2 *te = (float2 *)ctx->d_ew_te;
  YG_CUDA(cudaMemsetAsync(te + (size_t)N * lep, 0, (size_t)EW_MMA_TEPAD * lep * sizeof(float2), ctx->stream));
  k_tables_mma<<<yg_blocks(N, 32), 256, 0, ctx->stream>>>(ctx->d_pos, ctx->d_charge, N, ctx->cell, G0, G1, G2,
                                                          (float)qscale, lep, nmf, te, (uint2 *)ctx->d_ew_yf);
  YG_LAUNCH_CHECK(ctx, "k_tables_mma");
  if (usf) {
    if ((rc = yg_launch_yb_umma(ctx, ctx->d_ew_yf, lo, hi, gbase[1], gbase[2], ys_blocks, nmf, nks, ctx->d_ew_ys)))
      return rc;
  } else {
    k_ys_mma<<<yg_blocks(ys_blocks * nms * 8, 256), 256, 0, ctx->stream>>>(
        (const uint2 *)ctx->d_ew_yf, N, lo, hi, gbase[1], gbase[2], ys_blocks, nmf, nms, (uint4 *)ctx->d_ew_ys);
    YG_LAUNCH_CHECK(ctx, "k_ys_mma");
  }
  // structure factors: the warp-MMA S pass runs over conjugate column pairs
  // (128 partial columns per tile of 64 pairs)
  const bool pairs = !usf && YG_SFAC_PAIRS;
  const int stiles = pairs ? ctx->ew_ntp : ntile64, ssc = pairs ? 128 : 64;
  const int4 *scols = (const int4 *)(pairs ? ctx->d_ew_pcols : ctx->d_ew_tiles);
  const size_t ssm = 2 * ((size_t)EW_MMA_KS * lep * sizeof(float2) + (size_t)(EW_MMA_KS / 16) * nms * 8 * sizeof(uint4));
  const void *skern = pairs ? (const void *)k_sfac_mma<true> : (const void *)k_sfac_mma<false>;
  int sslots = 0;
  if (!usf) {
    if ((rc = yg_smem_optin(skern, ssm))) return rc;
    if ((rc = resident_blocks(skern, 128, ssm, &ctx->ew_occ_s, &sslots))) return rc;
  }
  // atoms per S-pass block: the fewest chunks whose blocks (chunks x tiles)
  // still fit one wave of resident blocks, at least EW_MMA_ATB, a multiple of
  // 32 (50,000 atoms on 17 pair tiles and 608 slots: 1,440 atoms, 35 x 17
  // blocks; one wave of 1,536-atom chunks measured 991 / 998 evals/s against
  // 976 / 979 for 1,024-atom chunks, 1.37 waves)
  auto chunk_of = [&](int64_t n) -> int {
    if (usf) return yg_umma_sfac_atb();
    const int64_t per_tile = std::max<int64_t>(1, sslots / std::max(1, stiles));
    int64_t a = (n + per_tile - 1) / per_tile;
    a = (a + 31) / 32 * 32;
    return (int)std::max<int64_t>(EW_MMA_ATB, a);
  };
  int maxchunk = 1;
  for (int g = 0; g < nS; g++) {
    const int64_t n = gb[g][1] - gb[g][0];
    if (n > 0) maxchunk = std::max(maxchunk, (int)((n + chunk_of(n) - 1) / chunk_of(n)));
  }
  const size_t per = (size_t)stiles * ssc * EW_MS;
  if ((rc = yg_ensure(ctx, &ctx->d_ew_Spart, &ctx->ew_bytes_Spart, per * maxchunk * sizeof(float2)))) return rc;
  for (int g = 0; g < nS; g++) {
    const int64_t n = gb[g][1] - gb[g][0];
    double *S = ctx->d_ew_S + (size_t)g * 2 * nk_dense;
    YG_CUDA(cudaMemsetAsync(S, 0, 2 * nk_dense * sizeof(double), ctx->stream));
    if (n <= 0) continue;
    const int atb = chunk_of(n);
    const int nch = (int)((n + atb - 1) / atb);
    if (usf) {
      if ((rc = yg_launch_sfac_umma(ctx, te + (size_t)gb[g][0] * lep,
                                    (const unsigned char *)ctx->d_ew_ys + (size_t)(gbase[g] / 16) * nks * 1024, (int)n,
                                    G0, lep, nks, ctx->d_ew_tiles, ctx->d_ew_Spart, ntile64, EW_MS)))
        return rc;
    } else {
      dim3 grid(nch, stiles, 1);
      auto kern = pairs ? k_sfac_mma<true> : k_sfac_mma<false>;
      kern<<<grid, 128, ssm, ctx->stream>>>(te + (size_t)gb[g][0] * lep,
                                            (const uint4 *)ctx->d_ew_ys + (size_t)(gbase[g] / 16) * nms * 8, (int)n,
                                            G0, lep, nms, scols, (float2 *)ctx->d_ew_Spart, stiles, 1, atb,
                                            ctx->d_status);
      YG_LAUNCH_CHECK(ctx, "k_sfac_mma");
    }
    k_sfac_reduce<float><<<yg_blocks((int64_t)per * 4, 256), 256, 0, ctx->stream>>>(
        (const float2 *)ctx->d_ew_Spart, nch, usf ? ntile64 : stiles, 1, usf ? 64 : ssc,
        usf ? (const int4 *)ctx->d_ew_tiles : scols, nm, 1.0 / qscale, S);
    YG_LAUNCH_CHECK(ctx, "k_sfac_reduce");
  }
  // energy, virial, weights of the force pass: B operands of the tcgen05
  // kernel, or fragments of the warp-level MMA kernel
  const int ngroup = (nS == 3) ? 3 : 1;
  const bool umma = want_grad && ctx->ew_umma && ctx->ew_force_path == 0;
  const int64_t wbstride = (int64_t)ctx->ew_wbunits * 256;  // 32-bit words per group
  const int64_t ubstride = (int64_t)ctx->ew_ubunits * 4096;  // 32-bit words per group
  if (umma) {
    if ((rc = yg_ensure(ctx, &ctx->d_ew_ub, &ctx->ew_bytes_ub, (size_t)ngroup * ubstride * 4))) return rc;
    YG_CUDA(cudaMemsetAsync(ctx->d_ew_ub, 0, (size_t)ngroup * ubstride * 4, ctx->stream));
  } else {
    if ((rc = yg_ensure(ctx, &ctx->d_ew_wb, &ctx->ew_bytes_wb, (size_t)ngroup * wbstride * 4))) return rc;
    YG_CUDA(cudaMemsetAsync(ctx->d_ew_wb, 0, (size_t)ngroup * wbstride * 4, ctx->stream));
  }
  const int eb = yg_blocks(nk_dense, 256);
  if ((rc = yg_ensure(ctx, (void **)&ctx->d_ew_red, &ctx->ew_red_cap, ((size_t)eb * 7 + 64 + 7) * sizeof(double))))
    return rc;
  double *partial = ctx->d_ew_red + 64;
  const double fac2 = 0.25 / ctx->ew_alpha / ctx->ew_alpha;
  k_ewald_energy<float><<<eb, 256, 0, ctx->stream>>>(
      ctx->d_ew_S, nS, nk_dense, ctx->d_ew_pref, G0, G1, nm, ctx->cell, fac2, ngroup, ctx->d_ew_wslot, 0, nullptr,
      umma ? nullptr : (unsigned *)ctx->d_ew_wb, ctx->d_ew_woff, wbstride, umma ? (unsigned *)ctx->d_ew_ub : nullptr,
      ctx->d_ew_uoff, ubstride, ctx->d_ew_uslot, s1, s2, partial);
  YG_LAUNCH_CHECK(ctx, "k_ewald_energy");
  double *sums = partial + (size_t)eb * 7;
  if ((rc = yg_launch_reduce_ev(ctx, partial, eb, 7, sums))) return rc;
  double *ev = ctx->d_part_ev + 10 * YG_PART_EWALD_RECI;
  k_store_ewald_ev<<<1, 32, 0, ctx->stream>>>(sums, 1.0 / ctx->ew_diel, ev);
  YG_LAUNCH_CHECK(ctx, "k_store_ewald_ev");
  double *gpos = ctx->d_part_gpos + (size_t)YG_PART_EWALD_RECI * N * 3;
  if (!want_grad) {
    YG_CUDA(cudaMemsetAsync(gpos, 0, N * 3 * sizeof(double), ctx->stream));
    ctx->part_valid[YG_PART_EWALD_RECI] = 1;
    return YG_OK;
  }
  // force pass, per atom group
  if ((rc = yg_ensure(ctx, (void **)&ctx->d_ew_gpart, &ctx->ew_bytes_gpart, (size_t)N * 3 * sizeof(double)))) return rc;
  if (umma) {
    // tcgen05: one CTA per SM (all of TMEM), blocks of 128 atoms x tile ranges
    int dev = 0, nsm = 1;
    YG_CUDA(cudaGetDevice(&dev));
    YG_CUDA(cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, dev));
    int64_t maxblk = 1;
    for (int g = 0; g < nS; g++) maxblk = std::max<int64_t>(maxblk, (gb[g][1] - gb[g][0] + 127) / 128);
    if ((rc = yg_ensure(ctx, &ctx->d_ew_ya, &ctx->ew_bytes_ya, (size_t)maxblk * nks * 2 * 4096))) return rc;
    for (int g = 0; g < nS; g++) {
      const int64_t n = gb[g][1] - gb[g][0];
      if (n <= 0) continue;
      const int nab = (int)((n + 127) / 128);
      if ((rc = yg_launch_ya_umma(ctx, ctx->d_ew_yf, gb[g][0], n, nmf, nks, nab, ctx->d_ew_ya))) return rc;
      // tile ranges per atom block: a CTA's time is its set-up (E0|E1 rows,
      // A operand, TMEM) plus its tiles (a K-step each and the epilogue), one
      // CTA per SM; the fewest ranges of the least estimated time
      const double tiles = (double)ctx->ew_ubunits + 4.0 * ctx->ew_nut, setup = YG_UMMA_SETUP;
      int nr = 1;
      double best = 1e300;
      for (int r = 1; r <= std::min(EW_MMA_MAXR, ctx->ew_nut); r++) {
        const double cost = std::ceil((double)nab * r / nsm) * (setup + tiles / r);
        if (cost < best * (1.0 - 1e-9)) {
          best = cost;
          nr = r;
        }
      }
      double *out = ctx->d_ew_gpart;
      const int64_t rstride = N * 3;
      if (nr > 1) {
        if ((rc = yg_ensure(ctx, (void **)&ctx->d_ew_fpiece, &ctx->ew_bytes_fpiece, (size_t)nr * rstride * sizeof(double))))
          return rc;
        out = ctx->d_ew_fpiece;
      }
      const void *ubg = (const unsigned *)ctx->d_ew_ub + (size_t)(ngroup == 1 ? 0 : g) * ubstride;
      if ((rc = yg_launch_force_umma(ctx, te, ctx->d_ew_ya, (int)gb[g][0], (int)gb[g][1], G0 + G1 + 2, G0, lep, nks,
                                     ctx->d_ew_urange + (nr - 1) * (nr + 2) / 2, nr, ubg, 1.0 / (qscale * s1),
                                     1.0 / (qscale * s2), out, rstride)))
        return rc;
      if (nr > 1) {
        k_ewald_force_mma_combine<<<yg_blocks(n * 3, 256), 256, 0, ctx->stream>>>(ctx->d_ew_fpiece, rstride, nr,
                                                                                  (int)gb[g][0], (int)gb[g][1],
                                                                                  ctx->d_ew_gpart);
        YG_LAUNCH_CHECK(ctx, "k_ewald_force_mma_combine");
      }
    }
    k_ewald_gpos<<<yg_blocks(N, 256), 256, 0, ctx->stream>>>(ctx->d_ew_gpart, N, ctx->cell,
                                                             -6.2831853071795864769 / ctx->ew_diel, gpos);
    YG_LAUNCH_CHECK(ctx, "k_ewald_gpos");
    ctx->part_valid[YG_PART_EWALD_RECI] = 1;
    return YG_OK;
  }
  const size_t fsm = (size_t)128 * lep * sizeof(float2) +
                     2 * ((size_t)EW_MMA_FT * nks * 1024 + EW_MMA_FT * 4 * sizeof(int4));
  if ((rc = yg_smem_optin((const void *)k_ewald_force_mma, fsm))) return rc;
  int slots;
  if ((rc = resident_blocks((const void *)k_ewald_force_mma, 256, fsm, &ctx->ew_occ_fm, &slots))) return rc;
  for (int g = 0; g < nS; g++) {
    const int64_t n = gb[g][1] - gb[g][0];
    if (n <= 0) continue;
    const uint4 *wbg = (const uint4 *)ctx->d_ew_wb + (size_t)(ngroup == 1 ? 0 : g) * (wbstride / 4);
    // column ranges: the count whose last wave is fullest (fewest on a tie)
    const int nab = (int)((n + 127) / 128);
    int nr = 1;
    double best = 0.0;
    for (int r = 1; r <= std::min(EW_MMA_MAXR, ctx->ew_nft4); r++) {
      const double waves = (double)nab * r / slots;
      const double eff = waves / std::ceil(waves);
      if (eff > best + 1e-9) {
        best = eff;
        nr = r;
      }
    }
    double *out = ctx->d_ew_gpart;
    const int64_t rstride = N * 3;
    if (nr > 1) {
      if ((rc = yg_ensure(ctx, (void **)&ctx->d_ew_fpiece, &ctx->ew_bytes_fpiece, (size_t)nr * rstride * sizeof(double))))
        return rc;
      out = ctx->d_ew_fpiece;
    }
    dim3 grid(nab, nr);
    k_ewald_force_mma<<<grid, 256, fsm, ctx->stream>>>(
        te, (const uint2 *)ctx->d_ew_yf, (int)gb[g][0], (int)gb[g][1], G0, lep, nmf, nks, (const int4 *)ctx->d_ew_tiles,
        ctx->d_ew_crange + (nr - 1) * (nr + 2) / 2, ctx->d_ew_woff, wbg, 1.0 / (qscale * s1), 1.0 / (qscale * s2),
        out, rstride, ctx->d_status);
    YG_LAUNCH_CHECK(ctx, "k_ewald_force_mma");
    if (nr > 1) {
      k_ewald_force_mma_combine<<<yg_blocks(n * 3, 256), 256, 0, ctx->stream>>>(ctx->d_ew_fpiece, rstride, nr,
                                                                                (int)gb[g][0], (int)gb[g][1],
                                                                                ctx->d_ew_gpart);
      YG_LAUNCH_CHECK(ctx, "k_ewald_force_mma_combine");
    }
  }
  k_ewald_gpos<<<yg_blocks(N, 256), 256, 0, ctx->stream>>>(ctx->d_ew_gpart, N, ctx->cell,
                                                           -6.2831853071795864769 / ctx->ew_diel, gpos);
  YG_LAUNCH_CHECK(ctx, "k_ewald_gpos");
  ctx->part_valid[YG_PART_EWALD_RECI] = 1;
  return YG_OK;
}
}  // namespace

// Host-side k-space layout: prefactor grid in the reference's formula and
// the list of 8x8 column tiles that intersect the half sphere.
int yg_launch_ewald_setup(yg_ctx *ctx) {
  int jrc;
  if ((jrc = yg_ewald_join(ctx))) return jrc;
  const int G0 = (int)ctx->ew_gmax[0], G1 = (int)ctx->ew_gmax[1], G2 = (int)ctx->ew_gmax[2];
  if (G2 + 1 > EW_MAXM) {
    yg_set_error("Ewald gmax[2] too large (G2+1 must be <= 64)");
    return YG_ERR_UNSUPPORTED;
  }
  const int nc0 = 2 * G0 + 1, nc1 = 2 * G1 + 1, nm = G2 + 1;
  const int64_t nk_dense = (int64_t)nc0 * nc1 * nm;
  std::vector<double> pref(nk_dense, 0.0);
  const double tp = 6.2831853071795864769, fp = 12.566370614359172954;
  double kv[9];
  for (int i = 0; i < 9; i++) kv[i] = tp * ctx->cell.gv[i];
  const double fac1 = fp / ctx->cell.volume;
  const double fac2 = 0.25 / ctx->ew_alpha / ctx->ew_alpha;
  double gc2 = ctx->ew_gcut * tp;
  gc2 *= gc2;
  int nk = 0;
  double amax = 0.0;
  std::vector<int> colmhi(nc0 * nc1, -1);
  for (int g0 = -G0; g0 <= G0; g0++)
    for (int g1 = -G1; g1 <= G1; g1++)
      for (int g2 = 0; g2 <= G2; g2++) {
        if (g2 == 0) {
          if (g1 < 0) continue;
          if (g1 == 0 && g0 <= 0) continue;
        }
        double k[3];
        k[0] = (g0 * kv[0] + g1 * kv[3] + g2 * kv[6]);
        k[1] = (g0 * kv[1] + g1 * kv[4] + g2 * kv[7]);
        k[2] = (g0 * kv[2] + g1 * kv[5] + g2 * kv[8]);
        double ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
        if (ksq > gc2) continue;
        int64_t col = (int64_t)(g0 + G0) * nc1 + (g1 + G1);
        pref[col * nm + g2] = fac1 * std::exp(-ksq * fac2) / ksq;
        amax = std::max(amax, pref[col * nm + g2]);
        if (g2 > colmhi[col]) colmhi[col] = g2;
        nk++;
      }
  // active columns sorted by decreasing extent, padded to a multiple of EW_SC
  std::vector<int4> tiles;
  for (int g0 = -G0; g0 <= G0; g0++)
    for (int g1 = -G1; g1 <= G1; g1++) {
      int64_t col = (int64_t)(g0 + G0) * nc1 + (g1 + G1);
      if (colmhi[col] >= 0) tiles.push_back(make_int4(g0, g1, (int)col, colmhi[col]));
    }
  std::stable_sort(tiles.begin(), tiles.end(), [](const int4 &x, const int4 &y) { return x.w > y.w; });
  while (tiles.size() % EW_SC) tiles.push_back(make_int4(0, 0, -1, -1));
  // conjugate column pairs: X(-g0, -g1) is the conjugate of X(g0, g1), so
  // the S pass forms one set of products per pair and the tcgen05 force pass
  // one P per pair.  Per pair the member with the larger extent comes first
  // ('+'), its partner (or padding) second; pairs sorted by that extent.
  const int4 pad = make_int4(0, 0, -1, -1);
  std::vector<std::pair<int4, int4>> pairs;
  {
    std::vector<char> used((size_t)nc0 * nc1, 0);
    for (const int4 &c : tiles) {
      if (c.z < 0 || used[c.z]) continue;
      used[c.z] = 1;
      int4 a = c, b = pad;
      if (c.x != 0 || c.y != 0) {
        const int64_t pc = (int64_t)(-c.x + G0) * nc1 + (-c.y + G1);
        if (colmhi[pc] >= 0 && !used[pc]) {
          used[pc] = 1;
          b = make_int4(-c.x, -c.y, (int)pc, colmhi[pc]);
          if (b.w > a.w) std::swap(a, b);
        }
      }
      pairs.push_back(std::make_pair(a, b));
    }
    std::stable_sort(pairs.begin(), pairs.end(),
                     [](const std::pair<int4, int4> &x, const std::pair<int4, int4> &y) { return x.first.w > y.first.w; });
  }
  // S pass (warp MMA): tiles of 64 pairs laid out as 64 '+' then 64 partners
  {
    const size_t ntp = (pairs.size() + 63) / 64;
    std::vector<int4> pcols(std::max<size_t>(1, ntp) * 128, pad);
    for (size_t q = 0; q < pairs.size(); q++) {
      pcols[(q / 64) * 128 + q % 64] = pairs[q].first;
      pcols[(q / 64) * 128 + 64 + q % 64] = pairs[q].second;
    }
    ctx->ew_ntp = (int)ntp;
    yg_free(ctx, (void **)&ctx->d_ew_pcols);
    ctx->d_ew_pcols = nullptr;
    int prc;
    if ((prc = yg_alloc(ctx, (void **)&ctx->d_ew_pcols, pcols.size() * sizeof(int4)))) return prc;
    YG_CUDA(cudaMemcpyAsync(ctx->d_ew_pcols, pcols.data(), pcols.size() * sizeof(int4), cudaMemcpyHostToDevice,
                            ctx->stream));
    YG_CUDA(cudaStreamSynchronize(ctx->stream));  // pcols goes out of scope
  }
  ctx->ew_ncol = nc0 * nc1;
  ctx->ew_nm = nm;
  ctx->ew_nk = nk;
  ctx->ew_ntile = (int)(tiles.size() / EW_SC);
  // force tiles (EW_FC columns each) that hold work, and the tiled-weight
  // slot of every dense column (-1: no k of the column is inside the cutoff)
  std::vector<int> wslot((size_t)nc0 * nc1, -1);
  int nft = 0;
  for (size_t i = 0; i < tiles.size(); i++) {
    if (tiles[i].z >= 0) wslot[tiles[i].z] = (int)i;
    if (i % EW_FC == 0 && tiles[i].w >= 0) nft++;
  }
  ctx->ew_nftile = nft;
  // force-pass cost of each column tile (its m extent plus the epilogue), as prefix sums
  std::vector<int> fpre(1, 0);
  for (int t = 0; t < nft; t++) fpre.push_back(fpre.back() + tiles[(size_t)t * EW_FC].w + 1 + EW_FEPI);
  yg_free(ctx, (void **)&ctx->d_ew_fpre);
  ctx->d_ew_fpre = nullptr;
  // tensor-core layout: 4-column tiles with work and their fragment units
  // (one 1 KB unit per 8 m values of the tile's extent)
  ctx->ew_amax = amax;
  // (the force pass stages 128 E0|E1 rows of G0 + G1 + 2 entries in shared memory)
  ctx->ew_mma = (nm <= 32 && G0 + G1 + 2 <= 160) ? 1 : 0;
  std::vector<int> woff(1, 0);
  for (size_t t = 0; t * 4 < tiles.size() && tiles[t * 4].w >= 0; t++) woff.push_back(woff.back() + (tiles[t * 4].w + 8) / 8);
  ctx->ew_nft4 = (int)woff.size() - 1;
  ctx->ew_wbunits = woff.back();
  // column ranges of the force pass for r = 1 .. EW_MMA_MAXR ranges, at
  // (r - 1)(r + 2) / 2: bounds of equal cost (6 MMAs per k-step plus an
  // epilogue worth about two)
  std::vector<int> crange;
  {
    std::vector<long long> cost(1, 0);
    for (int t = 0; t < ctx->ew_nft4; t++) cost.push_back(cost.back() + 6LL * (woff[t + 1] - woff[t]) + 2);
    for (int r = 1; r <= EW_MMA_MAXR; r++)
      for (int i = 0; i <= r; i++) {
        int t = 0;
        while (t < ctx->ew_nft4 && cost[t] * r < cost.back() * i) t++;
        crange.push_back(t);
      }
  }
  // tcgen05 force pass: 64-column tiles with work, their B-operand units (one
  // per 8 m values of the tile's extent) and tile ranges of equal cost
  // (three MMAs per K-step against an epilogue worth about four)
  // With YG_FORCE_PAIRS its 64-column tiles hold 32 conjugate pairs: the '+'
  // members in columns 0-31, their partners (or padding) in 32-63; the weights
  // of every column go to its slot of this list (uslot).
  const int ucols = yg_umma_cols();
  std::vector<int4> utiles;
  if (YG_FORCE_PAIRS) {
    const size_t half = ucols / 2, nt = (pairs.size() + half - 1) / half;
    utiles.assign(std::max<size_t>(1, nt) * ucols, pad);
    for (size_t q = 0; q < pairs.size(); q++) {
      utiles[(q / half) * ucols + q % half] = pairs[q].first;
      utiles[(q / half) * ucols + half + q % half] = pairs[q].second;
    }
  } else {
    utiles = tiles;
  }
  std::vector<int> uslot((size_t)nc0 * nc1, -1);
  for (size_t i = 0; i < utiles.size(); i++)
    if (utiles[i].z >= 0) uslot[utiles[i].z] = (int)i;
  std::vector<int> uoff(1, 0);
  for (size_t t = 0; t * ucols < utiles.size() && utiles[t * ucols].w >= 0; t++)
    uoff.push_back(uoff.back() + (utiles[t * ucols].w + 8) / 8);
  ctx->ew_nut = (int)uoff.size() - 1;
  ctx->ew_ubunits = uoff.back();
  ctx->ew_umma = (ctx->ew_mma && (nm + 7) / 8 <= yg_umma_kmax() && yg_umma_force_smem(G0 + G1 + 2) > 0) ? 1 : 0;
  std::vector<int> urange;
  {
    std::vector<long long> cost(1, 0);
    for (int t = 0; t < ctx->ew_nut; t++) cost.push_back(cost.back() + (uoff[t + 1] - uoff[t]) + 4);
    for (int r = 1; r <= EW_MMA_MAXR; r++)
      for (int i = 0; i <= r; i++) {
        int t = 0;
        while (t < ctx->ew_nut && cost[t] * r < cost.back() * i) t++;
        urange.push_back(t);
      }
  }
  yg_free(ctx, (void **)&ctx->d_ew_uoff);
  ctx->d_ew_uoff = nullptr;
  yg_free(ctx, (void **)&ctx->d_ew_upk);
  ctx->d_ew_upk = nullptr;
  yg_free(ctx, (void **)&ctx->d_ew_upf);
  ctx->d_ew_upf = nullptr;
  // every column of the tiles as one int for the tcgen05 epilogue: |g0|,
  // the E1 row G0 + 1 + |g1| (8 bits each), the signs of g0 and g1 (bits 16,
  // 17); -1 for padding
  std::vector<int> upk(std::max<size_t>(1, utiles.size()), -1);
  std::vector<float2> upf(std::max<size_t>(1, utiles.size()), make_float2(0.0f, 0.0f));
  for (size_t t = 0; t < utiles.size(); t++) {
    const int4 c = utiles[t];
    if (c.z >= 0) {
      upk[t] = std::abs(c.x) | ((G0 + 1 + std::abs(c.y)) << 8) | ((c.x < 0) << 16) | ((c.y < 0) << 17);
      upf[t] = make_float2((float)c.x, (float)c.y);
    }
  }
  yg_free(ctx, (void **)&ctx->d_ew_urange);
  ctx->d_ew_urange = nullptr;
  yg_free(ctx, (void **)&ctx->d_ew_crange);
  ctx->d_ew_crange = nullptr;
  yg_free(ctx, (void **)&ctx->d_ew_woff);
  ctx->d_ew_woff = nullptr;
  yg_free(ctx, (void **)&ctx->d_ew_wslot);
  yg_free(ctx, (void **)&ctx->d_ew_uslot);
  ctx->d_ew_uslot = nullptr;
  yg_free(ctx, (void **)&ctx->d_ew_pref);
  yg_free(ctx, (void **)&ctx->d_ew_tiles);
  yg_free(ctx, (void **)&ctx->d_ew_S);
  ctx->d_ew_pref = nullptr;
  ctx->d_ew_tiles = nullptr;
  ctx->d_ew_S = nullptr;
  int rc;
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_pref, nk_dense * sizeof(double)))) return rc;
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_tiles, std::max<size_t>(1, tiles.size()) * sizeof(int4)))) return rc;
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_S, 3 * 2 * nk_dense * sizeof(double)))) return rc;
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_wslot, wslot.size() * sizeof(int)))) return rc;
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_uslot, uslot.size() * sizeof(int)))) return rc;
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_uslot, uslot.data(), uslot.size() * sizeof(int), cudaMemcpyHostToDevice,
                          ctx->stream));
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_fpre, fpre.size() * sizeof(int)))) return rc;
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_woff, woff.size() * sizeof(int)))) return rc;
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_crange, crange.size() * sizeof(int)))) return rc;
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_uoff, uoff.size() * sizeof(int)))) return rc;
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_urange, urange.size() * sizeof(int)))) return rc;
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_upk, upk.size() * sizeof(int)))) return rc;
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_upk, upk.data(), upk.size() * sizeof(int), cudaMemcpyHostToDevice, ctx->stream));
  if ((rc = yg_alloc(ctx, (void **)&ctx->d_ew_upf, upf.size() * sizeof(float2)))) return rc;
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_upf, upf.data(), upf.size() * sizeof(float2), cudaMemcpyHostToDevice, ctx->stream));
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_uoff, uoff.data(), uoff.size() * sizeof(int), cudaMemcpyHostToDevice,
                          ctx->stream));
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_urange, urange.data(), urange.size() * sizeof(int), cudaMemcpyHostToDevice,
                          ctx->stream));
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_crange, crange.data(), crange.size() * sizeof(int), cudaMemcpyHostToDevice,
                          ctx->stream));
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_woff, woff.data(), woff.size() * sizeof(int), cudaMemcpyHostToDevice,
                          ctx->stream));
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_fpre, fpre.data(), fpre.size() * sizeof(int), cudaMemcpyHostToDevice,
                          ctx->stream));
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_wslot, wslot.data(), wslot.size() * sizeof(int), cudaMemcpyHostToDevice,
                          ctx->stream));
  YG_CUDA(cudaMemcpyAsync(ctx->d_ew_pref, pref.data(), nk_dense * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  if (!tiles.empty())
    YG_CUDA(cudaMemcpyAsync(ctx->d_ew_tiles, tiles.data(), tiles.size() * sizeof(int4), cudaMemcpyHostToDevice,
                            ctx->stream));
  YG_CUDA(cudaStreamSynchronize(ctx->stream));
  ctx->have_ewald = 1;
  return YG_OK;
}

int yg_ewald_join(yg_ctx *ctx) {
  if (ctx->ew_pending) {
    YG_CUDA(cudaStreamWaitEvent(ctx->stream, ctx->ew_join_ev, 0));
    ctx->ew_pending = 0;
  }
  return YG_OK;
}

static int launch_reci(yg_ctx *ctx, int want_grad);

// The reciprocal sum depends only on the positions, the charges and the
// k-space set-up, not on the neighbour list: it is forked onto the
// context's auxiliary stream so that it overlaps the neighbour build and the
// pair terms, and joined back by yg_ewald_join.
int yg_launch_ewald_reci(yg_ctx *ctx, int want_grad) {
  if (!ctx->ew_aux) {
    YG_CUDA(cudaStreamCreateWithFlags(&ctx->ew_aux, cudaStreamNonBlocking));
    YG_CUDA(cudaEventCreateWithFlags(&ctx->ew_fork_ev, cudaEventDisableTiming));
    YG_CUDA(cudaEventCreateWithFlags(&ctx->ew_join_ev, cudaEventDisableTiming));
  }
  YG_CUDA(cudaEventRecord(ctx->ew_fork_ev, ctx->stream));
  YG_CUDA(cudaStreamWaitEvent(ctx->ew_aux, ctx->ew_fork_ev, 0));
  cudaStream_t own = ctx->stream;
  ctx->stream = ctx->ew_aux;
  const int rc = launch_reci(ctx, want_grad);
  ctx->stream = own;
  YG_CUDA(cudaEventRecord(ctx->ew_join_ev, ctx->ew_aux));
  ctx->ew_pending = 1;
  return rc;
}

static int launch_reci(yg_ctx *ctx, int want_grad) {
  if (ctx->ew_ntile == 0) {
    double *ev = ctx->d_part_ev + 10 * YG_PART_EWALD_RECI;
    YG_CUDA(cudaMemsetAsync(ev, 0, 10 * sizeof(double), ctx->stream));
    YG_CUDA(cudaMemsetAsync(ctx->d_part_gpos + (size_t)YG_PART_EWALD_RECI * ctx->natom * 3, 0,
                            ctx->natom * 3 * sizeof(double), ctx->stream));
    ctx->part_valid[YG_PART_EWALD_RECI] = 1;
    return YG_OK;
  }
  if (ctx->precision == YG_FP64) return run_reci<double, double, 2>(ctx, want_grad);
  if (ctx->ew_mma) return run_reci_mma(ctx, want_grad);
  return run_reci<float, float, 2>(ctx, want_grad);
}

int yg_launch_ewald_corr(yg_ctx *ctx, int want_grad) {
  const int64_t N = ctx->natom;
  double *gpos = ctx->d_part_gpos + (size_t)YG_PART_EWALD_CORR * N * 3;
  YG_CUDA(cudaMemsetAsync(gpos, 0, N * 3 * sizeof(double), ctx->stream));
  // self term on the host, in the reference's order (ewald.c:289-292)
  extern double yg_host_self_energy(yg_ctx * ctx);
  double eself = yg_host_self_energy(ctx);
  const int64_t n = ctx->nstab;
  const int nb = yg_blocks(n > 0 ? n : 1, 256);
  int rc;
  if ((rc = yg_ensure(ctx, (void **)&ctx->d_red, &ctx->red_cap, ((size_t)nb * 7 + 64 + 7) * sizeof(double)))) return rc;
  double *partial = ctx->d_red + 64;
  k_ewald_corr<<<nb, 256, 0, ctx->stream>>>(ctx->d_pos, ctx->d_charge, ctx->d_stab_ab, ctx->d_stab_scale, n, ctx->cell,
                                            ctx->ew_alpha, ctx->ew_nlow, ctx->ew_nhigh, 1.0 / ctx->ew_diel,
                                            want_grad ? gpos : nullptr, partial);
  YG_LAUNCH_CHECK(ctx, "k_ewald_corr");
  double *sums = partial + (size_t)nb * 7;
  if ((rc = yg_launch_reduce_ev(ctx, partial, nb, 7, sums))) return rc;
  k_store_corr_ev<<<1, 32, 0, ctx->stream>>>(sums, eself / ctx->ew_diel, ctx->d_part_ev + 10 * YG_PART_EWALD_CORR);
  YG_LAUNCH_CHECK(ctx, "k_store_corr_ev");
  ctx->part_valid[YG_PART_EWALD_CORR] = 1;
  return YG_OK;
}
