// yg_ewald_umma.cu -- the two contractions of the mixed-precision reciprocal
// sum on the fifth-generation tensor cores (tcgen05.mma, accumulators in
// tensor memory): the force pass (below) and the structure-factor pass
// (k_sfac_umma, further down).
//
// The force on atom a from the reciprocal sum (yaff/pes/ewald.c:112-125,
// written as two contractions; see yg_ewald.cu) needs, per atom a and
// k-column c = (g0, g1):
//   Z_ac  = sum_m Y[a][m] U[c][m],   Z2_ac = sum_m m Y[a][m] U[c][m]
// (Y = q E2, U = conj of the weights 2 A(k) S_eff(k)), then the epilogue
//   grad_a += (g0 Im(P Z), g1 Im(P Z), Im(P Z2)),  P = E0[a][g0] E1[a][g1].
// Z and Z2 are one real GEMM per CTA and column tile:
//   D[128 atoms][256] = A[128 atoms][K] * B[K][256],
// K = 2 x (m values, re/im interleaved), the 256 output columns = 64 k-columns
// x (Z re, Z im, Z2 re, Z2 im).  Operands are FP16 hi + lo splits and each
// product is formed as hi*hi + hi*lo + lo*hi (about 22 significant bits);
// accumulation is FP32 in TMEM.  The tensor core's FP32 accumulation
// truncates toward zero; with at most 3 x 4 MMAs of K = 16 per accumulator the
// bias stays below 1e-6 of |Z|, as for the warp-level MMA form.
//
// Warp roles in a CTA of 576 threads (one CTA per SM, all 512 TMEM columns):
//   warp 0      bulk copies: the CTA's A operand once, then the B operand of
//               every tile into one of two stages (a stage is refilled once
//               the MMAs that read it have completed);
//   warp 1      allocates TMEM; one lane issues the MMAs of a tile into one
//               of two accumulators (256 columns each) and commits them to an
//               mbarrier;
//   warps 2-17  epilogue, four warps per TMEM lane quarter: warp w reads
//               lanes 32 (w % 4) .. + 31 (one atom per thread) of a quarter
//               of the tile's columns, forms P from the atom's E0|E1 row
//               (staged in shared memory transposed, so a column's reads
//               are conflict-free) and accumulates the three force
//               components; then releases the accumulator.  The four
//               partial sums of an atom are added in a fixed order at the
//               end.  The column list (g0, g1) of
//               a tile is read from global memory (one warp-uniform load per
//               column), not from a stage the producer may already refill.
// Shared-memory operands use the no-swizzle K-major layout: 8-row x 16-byte
// core matrices, the two K halves of a row group 128 B apart, row groups
// 256 B apart.  Every mbarrier wait is bounded (about a second); a wait that
// runs out records YG_ST_TIMEOUT and stops the CTA's roles, which then wait
// (bounded) for their own copies and MMAs still in flight before TMEM is
// freed and the CTA exits.
#include <cuda_fp16.h>

#include "yg_internal.cuh"

namespace {

constexpr int UM_M = 128;              // atoms per CTA (MMA M = TMEM lanes)
constexpr int UM_COLS = 64;            // k-columns per tile
constexpr int UM_N = 4 * UM_COLS;      // MMA N
constexpr int UM_KMAX = 4;             // K-steps (8 m values each) per tile, at most
constexpr int UM_ATILE = UM_M * 32;    // bytes of one A K-step half (128 rows x 16 FP16)
constexpr int UM_BTILE = UM_N * 32;    // bytes of one B K-step half (256 rows x 16 FP16)
constexpr int UM_EPI = 16;            // epilogue warps (four per TMEM lane quarter)
constexpr int UM_THREADS = 64 + 32 * UM_EPI;
constexpr int UM_TMEM_COLS = 2 * UM_N;
// instruction descriptor, kind::f16: D FP32 (bits 4-5 = 1), A and B FP16,
// both K-major, N >> 3 at bit 17, M >> 4 at bit 24
constexpr uint32_t UM_IDESC = (1u << 4) | ((uint32_t)(UM_N >> 3) << 17) | ((uint32_t)(UM_M >> 4) << 24);

constexpr size_t UM_SMEM_A = (size_t)UM_KMAX * 2 * UM_ATILE;   // 32 KB
constexpr size_t UM_SMEM_B = (size_t)UM_KMAX * 2 * UM_BTILE;   // 64 KB per stage

__device__ __forceinline__ unsigned um_smem(const void *p) { return (unsigned)__cvta_generic_to_shared(p); }

// shared-memory matrix descriptor: start >> 4, leading (K) byte offset 128,
// stride (8-row) byte offset `sbo`, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t um_desc_sbo(unsigned saddr, unsigned sbo) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
         ((uint64_t)1 << 46);
}
__device__ __forceinline__ uint64_t um_desc(unsigned saddr) { return um_desc_sbo(saddr, 256); }

__device__ __forceinline__ void um_mma_i(unsigned dtmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                         unsigned accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
      : "memory");
}
__device__ __forceinline__ void um_mma(unsigned dtmem, uint64_t adesc, uint64_t bdesc, unsigned accumulate) {
  um_mma_i(dtmem, adesc, bdesc, UM_IDESC, accumulate);
}

__device__ __forceinline__ void um_commit(unsigned long long *bar) {
  asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(um_smem(bar))
               : "memory");
}

__device__ __forceinline__ void um_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void um_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

__device__ __forceinline__ void um_ld32(unsigned taddr, float (&v)[32]) {
  unsigned r[32];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15,"
      "%16,%17,%18,%19,%20,%21,%22,%23,%24,%25,%26,%27,%28,%29,%30,%31}, [%32];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
        "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
        "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 32; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void um_ld16(unsigned taddr, float (&v)[16]) {
  unsigned r[16];
  asm volatile(
      "tcgen05.ld.sync.aligned.32x32b.x16.b32 {%0,%1,%2,%3,%4,%5,%6,%7,%8,%9,%10,%11,%12,%13,%14,%15}, [%16];"
      : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
        "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15])
      : "r"(taddr));
  asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory");
#pragma unroll
  for (int i = 0; i < 16; i++) v[i] = __uint_as_float(r[i]);
}

__device__ __forceinline__ void um_init(unsigned long long *bar, unsigned count) {
  asm volatile("mbarrier.init.shared::cta.b64 [%0], %1;" ::"r"(um_smem(bar)), "r"(count) : "memory");
}

__device__ __forceinline__ bool um_try(unsigned long long *bar, unsigned parity) {
  unsigned ok;
  asm volatile("{\n.reg .pred p;\nmbarrier.try_wait.parity.shared::cta.b64 p, [%1], %2;\nselp.u32 %0, 1, 0, p;\n}"
               : "=r"(ok)
               : "r"(um_smem(bar)), "r"(parity)
               : "memory");
  return ok != 0;
}

// Bounded wait for phase `parity`; gives up early when another role of the
// CTA gave up (*stop set), or after about a second (records the timeout and
// sets *stop).
__device__ __forceinline__ bool um_wait(unsigned long long *bar, unsigned parity, int *status, volatile int *stop) {
  for (int it = 0; it < (1 << 24); it++) {
    if (um_try(bar, parity)) return true;
    if ((it & 255) == 255 && *stop) return false;
  }
  if (status) atomicOr(status + YG_ST_TIMEOUT, 1);
  *stop = 1;
  return false;
}

// Bounded wait used when tearing down (ignores *stop).
__device__ __forceinline__ void um_drain(unsigned long long *bar, unsigned parity, int *status) {
  for (int it = 0; it < (1 << 24); it++)
    if (um_try(bar, parity)) return;
  if (status) atomicOr(status + YG_ST_TIMEOUT, 1);
}

__device__ __forceinline__ void um_expect(unsigned long long *bar, unsigned bytes) {
  unsigned long long state;
  asm volatile("mbarrier.arrive.expect_tx.shared::cta.b64 %0, [%1], %2;"
               : "=l"(state)
               : "r"(um_smem(bar)), "r"(bytes)
               : "memory");
}

__device__ __forceinline__ void um_copy(void *dst, const void *src, unsigned bytes, unsigned long long *bar) {
  asm volatile("cp.async.bulk.shared::cluster.global.mbarrier::complete_tx::bytes [%0], [%1], %2, [%3];" ::"r"(
                   um_smem(dst)),
               "l"(src), "r"(bytes), "r"(um_smem(bar))
               : "memory");
}

__device__ __forceinline__ void um_arrive(unsigned long long *bar) {
  unsigned long long state;
  asm volatile("mbarrier.arrive.shared::cta.b64 %0, [%1];" : "=l"(state) : "r"(um_smem(bar)) : "memory");
}

// Kahan-compensated FP32 sum.
struct UmAcc {
  float s, c;
  __device__ __forceinline__ void init() { s = c = 0.f; }
  __device__ __forceinline__ void add(float x) {
    const float y = x - c;
    const float t = s + y;
    c = (t - s) - y;
    s = t;
  }
};

// A operand of every 128-atom block of an atom group: per block and K-step
// (8 m values) two 4 KB halves (hi, lo) in the no-swizzle K-major layout.
// One thread per (block, K-step, row, K half): the row's 8 FP16 values are
// (re, im) of 4 consecutive m, i.e. 4 consecutive hi (or lo) words of yf.
// Rows past the group (or past the table's m range) are zero.
__global__ void k_ya_umma(const uint2 *__restrict__ yf, int64_t a0, int64_t n, int nmf, int nks, int64_t nblk,
                          uint4 *__restrict__ ya) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (u >= nblk * nks * UM_M * 2) return;
  const int h = (int)(u & 1);
  const int row = (int)((u >> 1) % UM_M);
  const int64_t rest = (u >> 1) / UM_M;
  const int ks = (int)(rest % nks);
  const int64_t blk = rest / nks;
  const int64_t r = blk * UM_M + row;
  uint4 hi = make_uint4(0u, 0u, 0u, 0u), lo = hi;
  if (r < n) {
    const uint2 *y = yf + (a0 + r) * nmf + 8 * ks + 4 * h;
    const uint2 y0 = y[0], y1 = y[1], y2 = y[2], y3 = y[3];
    hi = make_uint4(y0.x, y1.x, y2.x, y3.x);
    lo = make_uint4(y0.y, y1.y, y2.y, y3.y);
  }
  const int64_t base = (blk * nks + ks) * 2 * (UM_ATILE / 16);
  const int off = (row >> 3) * 16 + h * 8 + (row & 7);
  ya[base + off] = hi;
  ya[base + UM_ATILE / 16 + off] = lo;
}

// PAIR: the tile's columns 0-31 are the '+' members of conjugate pairs and
// 32-63 their partners (or padding, whose weights are zero); the partner of
// (g0, g1) is (-g0, -g1) with P' = conj P, so a pair adds
//   g0 (Im(P Z) - Im(conj P Z')), g1 (Im(P Z) - Im(conj P Z')),
//   Im(P Z2) + Im(conj P Z2')
// with P formed once; each epilogue warp takes one chunk of 8 pairs.
template <bool PAIR>
__global__ void __launch_bounds__(UM_THREADS, 1)
    k_ewald_force_umma(const float2 *__restrict__ te, const uint4 *__restrict__ ya, int a0, int a1, int ne, int G0,
                       int lep, int nks, const int *__restrict__ upk, const float2 *__restrict__ upf,
                       const int *__restrict__ urange,
                       const int *__restrict__ uoff, const uint4 *__restrict__ ub, double inv1, double inv2,
                       double *__restrict__ out, int64_t rstride, int *__restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem_um[];
  __shared__ __align__(8) unsigned long long bar_a, bar_b[2], bar_mma[2], bar_acc[2];
  __shared__ unsigned tmem_slot;
  __shared__ int stop_flag;
  volatile int *stop = &stop_flag;
  const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
  unsigned char *sA = smem_um;
  unsigned char *sB = smem_um + UM_SMEM_A;
  float2 *sE = reinterpret_cast<float2 *>(sB + 2 * UM_SMEM_B);
  const int u0 = urange[blockIdx.y], u1 = urange[blockIdx.y + 1];
  const int ntile = u1 - u0;
  const int bbase = a0 + blockIdx.x * UM_M;

  if (threadIdx.x == 0) {
    um_init(&bar_a, 1);
    for (int s = 0; s < 2; s++) {
      um_init(&bar_b[s], 1);
      um_init(&bar_mma[s], 1);
      um_init(&bar_acc[s], UM_EPI);
    }
    stop_flag = 0;
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (warp == 1) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(um_smem(&tmem_slot)),
                 "r"(UM_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  um_fence_before();
  __syncthreads();
  um_fence_after();
  const unsigned tmem = tmem_slot;

  if (warp == 0) {
    if (lane == 0) {
      um_expect(&bar_a, (unsigned)(nks * 2 * UM_ATILE));
      um_copy(sA, ya + (size_t)blockIdx.x * nks * 2 * (UM_ATILE / 16), (unsigned)(nks * 2 * UM_ATILE), &bar_a);
      int issued = 0;
      for (int i = 0; i < ntile; i++) {
        const int s = i & 1;
        // stage s is free once the MMAs of tile i - 2 have completed
        if (i >= 2 && !um_wait(&bar_mma[s], ((i >> 1) - 1) & 1, status, stop)) break;
        const int u = u0 + i;
        const int k0 = uoff[u], kn = uoff[u + 1] - k0;
        um_expect(&bar_b[s], (unsigned)(kn * 2 * UM_BTILE));
        um_copy(sB + s * UM_SMEM_B, ub + (size_t)k0 * (2 * UM_BTILE / 16), (unsigned)(kn * 2 * UM_BTILE), &bar_b[s]);
        issued = i + 1;
      }
      // every copy issued has landed before the CTA exits
      um_drain(&bar_a, 0, status);
      for (int i = (issued >= 2 ? issued - 2 : 0); i < issued; i++) um_drain(&bar_b[i & 1], (i >> 1) & 1, status);
    }
    __syncwarp();
  } else if (warp == 1) {
    if (lane == 0) {
      int committed = 0;
      if (um_wait(&bar_a, 0, status, stop)) {
        const unsigned aB = um_smem(sA);
        for (int i = 0; i < ntile; i++) {
          const int s = i & 1;
          if (!um_wait(&bar_b[s], (i >> 1) & 1, status, stop)) break;
          // the epilogue has released accumulator s (tile i - 2)
          if (!um_wait(&bar_acc[s], ((i >> 1) & 1) ^ 1, status, stop)) break;
          um_fence_after();
          const int u = u0 + i, kn = uoff[u + 1] - uoff[u];
          const unsigned d = tmem + (unsigned)(s * UM_N);
          const unsigned bB = um_smem(sB + s * UM_SMEM_B);
          for (int ks = 0; ks < kn; ks++) {
            const uint64_t ah = um_desc(aB + ks * 2 * UM_ATILE), al = um_desc(aB + ks * 2 * UM_ATILE + UM_ATILE);
            const uint64_t bh = um_desc(bB + ks * 2 * UM_BTILE), bl = um_desc(bB + ks * 2 * UM_BTILE + UM_BTILE);
            um_mma(d, ah, bh, ks > 0 ? 1u : 0u);
            um_mma(d, ah, bl, 1u);
            um_mma(d, al, bh, 1u);
          }
          um_commit(&bar_mma[s]);
          committed = i + 1;
        }
      }
      // the last MMAs have completed before TMEM is freed
      if (committed > 0) um_drain(&bar_mma[(committed - 1) & 1], ((committed - 1) >> 1) & 1, status);
    }
    __syncwarp();
  } else {
    // epilogue: UM_EPI warps, UM_EPI / 4 per TMEM lane quarter q (= warp % 4);
    // warp h of a quarter takes the 32-column chunks h, h + UM_EPI / 4, ...
    // of every tile; one atom per thread
    constexpr int HQ = UM_EPI / 4;
    const int q = warp & 3, h = (warp - 2) >> 2, r = 32 * q + lane;
    const float2 *row = te + (size_t)(bbase + r) * lep;
    for (int g = h; g < ne; g += HQ) sE[g * UM_M + r] = row[g];
    asm volatile("bar.sync 1, %0;" ::"n"(UM_EPI * 32) : "memory");
    UmAcc acc0, acc1, acc2;
    acc0.init();
    acc1.init();
    acc2.init();
    // the packed columns of the next chunk (8 ints) are loaded while the
    // current chunk is worked on; after a tile's last chunk, the next tile's
    // first (the table is static, so loading ahead of the MMAs is safe)
    int4 na = make_int4(-1, -1, -1, -1), nb = na;
    if (ntile > 0) {
      const int4 *p = reinterpret_cast<const int4 *>(upk + (size_t)u0 * UM_COLS + 8 * h);
      na = __ldg(p);
      nb = __ldg(p + 1);
    }
    for (int i = 0; i < ntile; i++) {
      const int s = i & 1;
      if (!um_wait(&bar_mma[s], (i >> 1) & 1, status, stop)) break;
      um_fence_after();
      const unsigned tb = tmem + ((unsigned)(32 * q) << 16) + (unsigned)(s * UM_N);
      float p0 = 0.f, p1 = 0.f, p2 = 0.f;
      if (PAIR) {
        // pair chunk h: '+' columns 8 h .. 8 h + 7 (TMEM chunk h), partners
        // 32 + 8 h .. (chunk h + 4); four pairs at a time
        const int4 ca = na, cb = nb;
        if (i + 1 < ntile) {
          const int4 *p = reinterpret_cast<const int4 *>(upk + (size_t)(u0 + i + 1) * UM_COLS + 8 * h);
          na = __ldg(p);
          nb = __ldg(p + 1);
        }
        if (ca.x >= 0) {
          const float4 *fp = reinterpret_cast<const float4 *>(upf + (size_t)(u0 + i) * UM_COLS + 8 * h);
          const int pk[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
#pragma unroll
          for (int sub = 0; sub < 2; sub++) {
            const float4 f0 = __ldg(fp + 2 * sub), f1 = __ldg(fp + 2 * sub + 1);
            const float gf[8] = {f0.x, f0.y, f0.z, f0.w, f1.x, f1.y, f1.z, f1.w};
            float v[16], w[16];
            um_ld16(tb + 32 * h + 16 * sub, v);
            um_ld16(tb + 32 * (h + 4) + 16 * sub, w);
#pragma unroll
            for (int jj = 0; jj < 4; jj++) {
              const int col = pk[4 * sub + jj];
              if (col >= 0) {
                const int ag0 = col & 255, ag1 = (col >> 8) & 255;
                const bool n0 = (col >> 16) & 1, n1 = (col >> 17) & 1;
                const float2 e0 = sE[ag0 * UM_M + r], e1 = sE[ag1 * UM_M + r];
                const float e0y = n0 ? -e0.y : e0.y, e1y = n1 ? -e1.y : e1.y;
                const float pr = e0.x * e1.x - e0y * e1y;
                const float pi = e0.x * e1y + e0y * e1.x;
                const float im1 = pr * v[4 * jj + 1] + pi * v[4 * jj];
                const float im2 = pr * v[4 * jj + 3] + pi * v[4 * jj + 2];
                const float jm1 = pr * w[4 * jj + 1] - pi * w[4 * jj];
                const float jm2 = pr * w[4 * jj + 3] - pi * w[4 * jj + 2];
                const float d1 = im1 - jm1;
                p0 += gf[2 * jj] * d1;
                p1 += gf[2 * jj + 1] * d1;
                p2 += im2 + jm2;
              }
            }
          }
        }
      }
#pragma unroll 1
      for (int c = h; !PAIR && c < UM_N / 32; c += HQ) {
        const int4 ca = na, cb = nb;
        const bool last = c + HQ >= UM_N / 32 || ca.x < 0;  // (padding: the rest of the tile is padding)
        if (!last || i + 1 < ntile) {
          const int4 *p = reinterpret_cast<const int4 *>(
              upk + (size_t)(u0 + (last ? i + 1 : i)) * UM_COLS + 8 * (last ? h : c + HQ));
          na = __ldg(p);
          nb = __ldg(p + 1);
        }
        if (ca.x < 0) break;
        // the chunk's signed (g0, g1) as floats (the same for every lane)
        float gf[16];
        {
          const float4 *fp = reinterpret_cast<const float4 *>(upf + (size_t)(u0 + i) * UM_COLS + 8 * c);
#pragma unroll
          for (int k = 0; k < 4; k++) {
            const float4 f = __ldg(fp + k);
            gf[4 * k] = f.x;
            gf[4 * k + 1] = f.y;
            gf[4 * k + 2] = f.z;
            gf[4 * k + 3] = f.w;
          }
        }
        float v[32];
        um_ld32(tb + 32 * c, v);
        const int pk[8] = {ca.x, ca.y, ca.z, ca.w, cb.x, cb.y, cb.z, cb.w};
#pragma unroll
        for (int jj = 0; jj < 8; jj++) {
          const int col = pk[jj];
          if (col >= 0) {
            const int ag0 = col & 255, ag1 = (col >> 8) & 255;
            const bool n0 = (col >> 16) & 1, n1 = (col >> 17) & 1;
            const float2 e0 = sE[ag0 * UM_M + r], e1 = sE[ag1 * UM_M + r];
            const float e0y = n0 ? -e0.y : e0.y, e1y = n1 ? -e1.y : e1.y;
            const float pr = e0.x * e1.x - e0y * e1y;
            const float pi = e0.x * e1y + e0y * e1.x;
            const float im1 = pr * v[4 * jj + 1] + pi * v[4 * jj];
            const float im2 = pr * v[4 * jj + 3] + pi * v[4 * jj + 2];
            p0 += gf[2 * jj] * im1;
            p1 += gf[2 * jj + 1] * im1;
            p2 += im2;
          }
        }
      }
      um_fence_before();
      __syncwarp();
      if (lane == 0) um_arrive(&bar_acc[s]);
      acc0.add(p0);
      acc1.add(p1);
      acc2.add(p2);
    }
    // the HQ partial sums of every atom, added in a fixed order; the stage
    // buffers are idle now (the MMAs consumed every copy), so they hold them
    double *red = reinterpret_cast<double *>(sB);
    red[((size_t)h * UM_M + r) * 3 + 0] = (double)acc0.s;
    red[((size_t)h * UM_M + r) * 3 + 1] = (double)acc1.s;
    red[((size_t)h * UM_M + r) * 3 + 2] = (double)acc2.s;
    asm volatile("bar.sync 1, %0;" ::"n"(UM_EPI * 32) : "memory");
    const int a = bbase + r;
    if (h == 0 && a < a1) {
      double t0 = 0.0, t1 = 0.0, t2 = 0.0;
      for (int hh = 0; hh < HQ; hh++) {
        t0 += red[((size_t)hh * UM_M + r) * 3 + 0];
        t1 += red[((size_t)hh * UM_M + r) * 3 + 1];
        t2 += red[((size_t)hh * UM_M + r) * 3 + 2];
      }
      double *dst = out + (int64_t)blockIdx.y * rstride + (int64_t)a * 3;
      dst[0] = t0 * inv1;
      dst[1] = t1 * inv1;
      dst[2] = t2 * inv2;
    }
  }
  um_fence_before();
  __syncthreads();
  if (warp == 1) {
    um_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(UM_TMEM_COLS) : "memory");
  }
}

// ---------------------------------------------------------------------------
// S pass on tcgen05: the structure-factor partials of one chunk of atoms and
// one tile of 64 k-columns,
//   S[c][m] = sum_a X[a][c] Y[a][m],  X = E0[a][g0] E1[a][g1],  Y = q E2[a][m],
// as the real product D[128][N] = A[128][K] B[K][N] over K = atoms:
// A rows 0-63 are Re X of the tile's columns, rows 64-127 Im X; the N = 16 j
// columns of B are j groups of 16 (Re Y of 8 m values, then Im Y of the
// same 8), j = ceil(extent / 8) for the tile's largest m extent.  Then
//   Re S = D[c][Re Y] - D[c + 64][Im Y],  Im S = D[c][Im Y] + D[c + 64][Re Y].
// Operands are FP16 hi + lo splits, each product hi*hi + hi*lo + lo*hi.
//
// Warps 0-7 form X for a stage of 32 atoms (thread = one k-column and 8
// atoms: both rows, hi and lo, four 16-byte stores) into one of two A
// buffers, from the atoms' E0|E1 rows (a ring of three stages filled by
// bulk copies); warp 8 (one lane) issues the copies and, after the stage's
// barrier, waits for the stage's B operand (a ring of four) and issues its
// six MMAs into one of three 64-column TMEM accumulators, from zero, then
// commits them.  The X warps read an accumulator back two stages later (each
// warp its TMEM lane quarter, the two warp halves alternate 16-column
// groups) into FP32 registers with round-to-nearest, so the tensor core's
// truncating accumulation spans six MMAs (32 atoms) and the MMAs of two
// stages overlap the X formation.  (Twelve MMAs per accumulator, 64 atoms,
// biased |S| low enough to move the energy of a 3,000-atom box by 3.5e-7
// relative.)  The warp-level MMA form measured faster (183 against 218 us at
// 50,000 atoms: both are bound by the CUDA-core X formation, which this form
// also stores to shared memory and synchronises), so it is the automatic
// choice and this kernel is selected with yg_ewald_sfac_path(ctx, 2).  One CTA barrier per stage; every other
// dependency is an mbarrier: E rows landed (X warps), B landed and MMAs
// complete (warp 8 before refilling a B stage; the X warps before reusing an
// A buffer or reading an accumulator).  Padding columns (past the sorted
// list) get finite X and their partials are never read.  At the end the
// sums go through shared memory (rows padded to 65 words) to the partial
// S[chunk][tile][c][m] (row stride sms).
//
// Operand layout (no swizzle, K-major): 8-row x 16-byte core matrices, the
// two 8-atom halves of a K-step 128 B apart, the hi part of a row group at
// +0 and its lo part at +256, row groups 512 B apart.  A: 8 KB per K-step
// (16 row groups); B: 1 KB per 8 m values per K-step (two row groups), the
// Y operand of a 16-atom block stored as nks KB in that layout (k_yb_umma).
// Waits are bounded; a wait that runs out records YG_ST_TIMEOUT, all
// threads leave the loop together at the next barrier, and warp 8 waits
// (bounded) for the copies and MMAs still in flight before TMEM is freed.

#ifndef YG_SFAC_ATB
#define YG_SFAC_ATB 512   // atoms per CTA (a multiple of 32)
#endif
#ifndef YG_SFAC_MINB
#define YG_SFAC_MINB 2    // resident CTAs per SM the register budget is sized for
#endif

constexpr int US_XW = 8;                       // X-forming warps
constexpr int US_THREADS = 32 * (US_XW + 1);   // + the copy/MMA warp
constexpr int US_KS = 32;                      // atoms per stage (two K-steps)
constexpr int US_NT = 3;                       // E-row stages
constexpr int US_NB = 4;                       // B stages
constexpr int US_NACC = 3;                     // TMEM accumulators of 64 columns
constexpr int US_ABYTES = 2 * 8192;            // A operand of a stage
constexpr int US_BBYTES = 2 * 4096;            // B operand of a stage (at most four 8-m groups)
constexpr int US_TMEM_COLS = 256;
constexpr int US_DSTRIDE = 65;                 // words per row of the final D staging

__device__ __forceinline__ unsigned um_h2(__half2 h) { return *reinterpret_cast<unsigned *>(&h); }

// (a, b) -> FP16 pairs hi = rn(a, b), lo = rn(a - hi, b - hi).
__device__ __forceinline__ void um_split(float a, float b, unsigned &hi, unsigned &lo) {
  const __half2 h = __floats2half2_rn(a, b);
  const float2 f = __half22float2(h);
  hi = um_h2(h);
  lo = um_h2(__floats2half2_rn(a - f.x, b - f.y));
}

// Bounded wait without a stop flag (every waiting thread polls itself).
__device__ __forceinline__ bool um_wait_all(unsigned long long *bar, unsigned parity, int *status) {
  for (int it = 0; it < (1 << 24); it++)
    if (um_try(bar, parity)) return true;
  if (status) atomicOr(status + YG_ST_TIMEOUT, 1);
  return false;
}

// B operand of the S pass: per 16-atom block (positions relative to the atom
// groups as in the warp-MMA form: [lo, hi), [0, lo), [hi, N), each padded to
// whole blocks; padding atoms read zero) nks KB; one thread per 16-byte unit
// (block, row group gi = 2 (m / 8) + (0 re, 1 im), hi/lo, 8-atom half, row
// m % 8) packs the FP16 values of 8 atoms.
__global__ void k_yb_umma(const uint2 *__restrict__ yf, int64_t lo, int64_t hi, int64_t natom, int64_t base1,
                          int64_t base2, int64_t nblocks, int nmf, int nks, uint4 *__restrict__ yb) {
  const int64_t u = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  const int64_t per = (int64_t)nks * 64;
  if (u >= nblocks * per) return;
  const int r = (int)(u & 7), kh = (int)((u >> 3) & 1), hl = (int)((u >> 4) & 1);
  const int gi = (int)((u % per) >> 5);
  const int64_t blk = u / per;
  const int m = 8 * (gi >> 1) + r, comp = gi & 1;
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
#pragma unroll
  for (int k = 0; k < 8; k++) {
    const int64_t rr = p0 + 8 * kh + k - gbase;
    unsigned h16 = 0u;
    if (rr >= 0 && rr < n && m < nmf) {
      const uint2 v = yf[(a0 + rr) * nmf + m];
      const unsigned half2 = hl ? v.y : v.x;
      h16 = comp ? (half2 >> 16) : (half2 & 0xffffu);
    }
    w[k >> 1] |= h16 << (16 * (k & 1));
  }
  yb[blk * per + gi * 32 + hl * 16 + kh * 8 + r] = make_uint4(w[0], w[1], w[2], w[3]);
}

__global__ void __launch_bounds__(US_THREADS, YG_SFAC_MINB)
    k_sfac_umma(const float2 *__restrict__ te, const uint4 *__restrict__ yb, int n, int G0, int lep, int nks,
                const int4 *__restrict__ cols, float2 *__restrict__ Spart, int ntile64, int sms,
                int *__restrict__ status) {
  extern __shared__ __align__(1024) unsigned char smem_us[];
  __shared__ __align__(8) unsigned long long bar_te[US_NT], bar_b[US_NB], bar_mma[2];
  __shared__ unsigned tmem_slot;
  const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
  const bool ctl = warp == US_XW;
  const int tile = blockIdx.y;
  const int extent = cols[tile * 64].w + 1;  // columns sorted by decreasing extent
  const int j = extent > 0 ? (extent + 7) >> 3 : 0;
  const int abeg = blockIdx.x * YG_SFAC_ATB, aend = min(n, abeg + YG_SFAC_ATB);
  if (j == 0 || aend <= abeg) return;  // whole CTA, before any barrier or TMEM
  const unsigned te_bytes = (unsigned)(US_KS * lep * sizeof(float2));
  unsigned char *sA = smem_us;                          // 2 x US_ABYTES
  unsigned char *sT = smem_us + 2 * US_ABYTES;          // US_NT x te_bytes
  unsigned char *sB = sT + (size_t)US_NT * te_bytes;    // US_NB x US_BBYTES
  const uint32_t idesc = (1u << 4) | ((uint32_t)(2 * j) << 17) | ((uint32_t)(128 >> 4) << 24);
  const int nst = (aend - abeg + US_KS - 1) / US_KS;
  // this X thread's k-column and 8-atom slice of a stage
  const int c = tid & 63, hk = (tid >> 6) & 3, ks_t = hk >> 1, kh_t = hk & 1;
  int o0 = 0, o1 = 0;
  float s0 = 1.f, s1 = 1.f;
  if (!ctl) {
    const int4 col = cols[tile * 64 + c];
    o0 = col.x < 0 ? -col.x : col.x;
    o1 = G0 + 1 + (col.y < 0 ? -col.y : col.y);
    s0 = col.x < 0 ? -1.f : 1.f;
    s1 = col.y < 0 ? -1.f : 1.f;
  }
  if (tid == 0) {
    for (int i = 0; i < US_NT; i++) um_init(&bar_te[i], 1);
    for (int i = 0; i < US_NB; i++) um_init(&bar_b[i], 1);
    um_init(&bar_mma[0], 1);
    um_init(&bar_mma[1], 1);
    asm volatile("fence.mbarrier_init.release.cluster;" ::: "memory");
  }
  if (ctl) {
    asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(um_smem(&tmem_slot)),
                 "r"(US_TMEM_COLS)
                 : "memory");
    asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
  }
  um_fence_before();
  __syncthreads();
  um_fence_after();
  const unsigned tmem = tmem_slot;
  // copies (warp 8, lane 0): E rows of atoms abeg + 32 s .. + 31 (te holds
  // zero rows past the last atom), B operand of the stage's two 16-atom blocks
  auto issue_te = [&](int s) {
    const int b = s % US_NT;
    um_expect(&bar_te[b], te_bytes);
    um_copy(sT + (size_t)b * te_bytes, te + (size_t)(abeg + s * US_KS) * lep, te_bytes, &bar_te[b]);
  };
  auto issue_b = [&](int s) {
    const int b = s % US_NB;
    unsigned char *dst = sB + (size_t)b * US_BBYTES;
    const uint4 *src = yb + (size_t)((abeg + s * US_KS) / 16) * nks * 64;
    um_expect(&bar_b[b], 2048u * (unsigned)j);
    um_copy(dst, src, 1024u * (unsigned)j, &bar_b[b]);
    um_copy(dst + 4096, src + (size_t)nks * 64, 1024u * (unsigned)j, &bar_b[b]);
  };
  const bool leader = ctl && lane == 0;
  int te_issued = 0, b_issued = 0, b_waited = 0, committed = 0;  // (leader's bookkeeping)
  if (leader) {
    for (; te_issued < min(nst, US_NT); te_issued++) issue_te(te_issued);
    for (; b_issued < min(nst, US_NB); b_issued++) issue_b(b_issued);
  }
  float acc[2][16];
#pragma unroll
  for (int t = 0; t < 2; t++)
#pragma unroll
    for (int e = 0; e < 16; e++) acc[t][e] = 0.f;
  const int q = warp & 3, hh = (warp >> 2) & 1;
  const unsigned tl = tmem + ((unsigned)(32 * q) << 16);
  auto readback = [&](int slot) {
#pragma unroll
    for (int t = 0; t < 2; t++) {
      const int i = hh + 2 * t;
      if (i < j) {
        float v[16];
        um_ld16(tl + (unsigned)(slot * 64 + 16 * i), v);
#pragma unroll
        for (int e = 0; e < 16; e++) acc[t][e] += v[e];
      }
    }
  };
  bool fail = false;
  int s = 0;
  for (; s < nst; s++) {
    if (!ctl) {
      if (!um_wait_all(&bar_te[s % US_NT], (unsigned)((s / US_NT) & 1), status)) fail = true;
      if (!fail && s >= 2) {
        // the MMAs of stage s - 2 are complete: A buffer s & 1 is free and
        // accumulator (s - 2) % 3 holds that stage's sums
        if (!um_wait_all(&bar_mma[s & 1], (unsigned)(((s - 2) >> 1) & 1), status)) {
          fail = true;
        } else {
          um_fence_after();
          readback((s - 2) % US_NACC);
          um_fence_before();
        }
      }
      const int nrow = min(US_KS, aend - (abeg + s * US_KS));
      if (!fail && 16 * ks_t < nrow) {
        const float2 *row =
            reinterpret_cast<const float2 *>(sT + (size_t)(s % US_NT) * te_bytes) + (size_t)(16 * ks_t + 8 * kh_t) * lep;
        unsigned xrh[4], xrl[4], xih[4], xil[4];
#pragma unroll
        for (int i = 0; i < 4; i++) {
          float xr[2], xi[2];
#pragma unroll
          for (int u = 0; u < 2; u++) {
            const float2 *ra = row + (size_t)(2 * i + u) * lep;
            const float2 e0 = ra[o0], e1 = ra[o1];
            const float e0y = e0.y * s0, e1y = e1.y * s1;
            xr[u] = e0.x * e1.x - e0y * e1y;
            xi[u] = e0.x * e1y + e0y * e1.x;
          }
          um_split(xr[0], xr[1], xrh[i], xrl[i]);
          um_split(xi[0], xi[1], xih[i], xil[i]);
        }
        unsigned char *A = sA + (size_t)(s & 1) * US_ABYTES + ks_t * 8192 + kh_t * 128 + (c & 7) * 16 + (c >> 3) * 512;
        *reinterpret_cast<uint4 *>(A) = make_uint4(xrh[0], xrh[1], xrh[2], xrh[3]);
        *reinterpret_cast<uint4 *>(A + 256) = make_uint4(xrl[0], xrl[1], xrl[2], xrl[3]);
        *reinterpret_cast<uint4 *>(A + 4096) = make_uint4(xih[0], xih[1], xih[2], xih[3]);
        *reinterpret_cast<uint4 *>(A + 4096 + 256) = make_uint4(xil[0], xil[1], xil[2], xil[3]);
      }
      asm volatile("fence.proxy.async.shared::cta;" ::: "memory");
    }
    um_fence_before();
    if (__syncthreads_or(fail)) break;
    um_fence_after();
    if (leader) {
      // E-row stage s % 3 is consumed: refill it
      if (te_issued < nst) issue_te(te_issued++);
      // the MMAs of stage s - 2 are complete: refill its B stage
      if (s >= 2 && b_issued < nst) {
        if (!um_wait_all(&bar_mma[s & 1], (unsigned)(((s - 2) >> 1) & 1), status)) fail = true;
        else issue_b(b_issued++);
      }
      if (!fail && !um_wait_all(&bar_b[s % US_NB], (unsigned)((s / US_NB) & 1), status)) fail = true;
      if (!fail) {
        b_waited = s + 1;
        um_fence_after();
        const int nkv = min(US_KS, aend - (abeg + s * US_KS)) > 16 ? 2 : 1;
        const unsigned aB = um_smem(sA + (size_t)(s & 1) * US_ABYTES);
        const unsigned bB = um_smem(sB + (size_t)(s % US_NB) * US_BBYTES);
        const unsigned d = tmem + (unsigned)((s % US_NACC) * 64);
        for (int ks = 0; ks < nkv; ks++) {
          const uint64_t ah = um_desc_sbo(aB + ks * 8192, 512), al = um_desc_sbo(aB + ks * 8192 + 256, 512);
          const uint64_t bh = um_desc_sbo(bB + ks * 4096, 512), bl = um_desc_sbo(bB + ks * 4096 + 256, 512);
          um_mma_i(d, ah, bh, idesc, ks > 0 ? 1u : 0u);
          um_mma_i(d, ah, bl, idesc, 1u);
          um_mma_i(d, al, bh, idesc, 1u);
        }
        um_commit(&bar_mma[s & 1]);
        committed = s + 1;
      }
    }
  }
  if (!fail && !ctl) {
    // the last two stages' sums
    for (int t = max(0, nst - 2); t < nst && !fail; t++) {
      if (!um_wait_all(&bar_mma[t & 1], (unsigned)((t >> 1) & 1), status)) {
        fail = true;
      } else {
        um_fence_after();
        readback(t % US_NACC);
        um_fence_before();
      }
    }
  }
  fail = __syncthreads_or(fail);
  if (fail) {
    // copies and MMAs still in flight land before the buffers and TMEM go:
    // E-row stages from the one the loop stopped at, B stages the leader had
    // not waited for, the MMAs up to the last commit (one outstanding phase
    // per barrier, so each parity is unambiguous)
    if (leader) {
      for (int t = min(s, te_issued); t < te_issued; t++)
        um_drain(&bar_te[t % US_NT], (unsigned)((t / US_NT) & 1), status);
      for (int t = b_waited; t < b_issued; t++) um_drain(&bar_b[t % US_NB], (unsigned)((t / US_NB) & 1), status);
      if (committed > 0) um_drain(&bar_mma[(committed - 1) & 1], (unsigned)(((committed - 1) >> 1) & 1), status);
    }
  } else {
    // D rows through shared memory (A and E-row buffers are idle: every copy
    // was consumed and every MMA has completed)
    float *Dsm = reinterpret_cast<float *>(smem_us);
    if (!ctl) {
      const int L = 32 * q + lane;
#pragma unroll
      for (int t = 0; t < 2; t++) {
        const int i = hh + 2 * t;
        if (i < j) {
#pragma unroll
          for (int e = 0; e < 16; e++) Dsm[L * US_DSTRIDE + 16 * i + e] = acc[t][e];
        }
      }
    }
    __syncthreads();
    const int nmv = 8 * j;
    float2 *dst = Spart + ((int64_t)blockIdx.x * ntile64 + tile) * 64 * sms;
    for (int idx = tid; idx < 64 * nmv; idx += US_THREADS) {
      const int cc = idx / nmv, m = idx - cc * nmv;
      const int cre = 16 * (m >> 3) + (m & 7), cim = cre + 8;
      const float *dr = Dsm + cc * US_DSTRIDE, *di = Dsm + (cc + 64) * US_DSTRIDE;
      dst[(int64_t)cc * sms + m] = make_float2(dr[cre] - di[cim], dr[cim] + di[cre]);
    }
  }
  um_fence_before();
  __syncthreads();
  if (ctl) {
    um_fence_after();
    asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(US_TMEM_COLS) : "memory");
  }
}

}  // namespace

// Dynamic shared memory of the tcgen05 force pass for ne E0|E1 entries per
// atom; 0 when it does not fit on a multiprocessor.
size_t yg_umma_force_smem(int ne) {
  const size_t need = UM_SMEM_A + 2 * UM_SMEM_B + (size_t)ne * UM_M * sizeof(float2);
  return need <= 225 * 1024 ? need : 0;
}

int yg_umma_kmax() { return UM_KMAX; }
int yg_umma_cols() { return UM_COLS; }

// Dynamic shared memory of the tcgen05 S pass for E0|E1 rows of lep float2
// (lep even); 0 when two CTAs do not fit on a multiprocessor (228 KB, less
// 1 KB reserved and 1 KB of static shared memory per CTA).
size_t yg_umma_sfac_smem(int lep) {
  const size_t need = 2 * (size_t)US_ABYTES + (size_t)US_NT * US_KS * lep * sizeof(float2) + (size_t)US_NB * US_BBYTES;
  return (lep % 2 == 0 && need <= 112 * 1024) ? need : 0;
}
int yg_umma_sfac_atb() { return YG_SFAC_ATB; }

// B operand of the tcgen05 S pass (nblocks 16-atom blocks, nks KB each).
int yg_launch_yb_umma(yg_ctx *ctx, const void *yf, int64_t lo, int64_t hi, int64_t base1, int64_t base2,
                      int64_t nblocks, int nmf, int nks, void *yb) {
  const int64_t threads = nblocks * nks * 64;
  if (threads <= 0) return YG_OK;
  k_yb_umma<<<yg_blocks(threads, 256), 256, 0, ctx->stream>>>((const uint2 *)yf, lo, hi, ctx->natom, base1, base2,
                                                              nblocks, nmf, nks, (uint4 *)yb);
  YG_LAUNCH_CHECK(ctx, "k_yb_umma");
  return YG_OK;
}

// Structure-factor partials of the n atoms of one group (te, yb start at the
// group) over ntile64 column tiles: Spart[chunk][tile][c][m], row stride sms.
int yg_launch_sfac_umma(yg_ctx *ctx, const void *te, const void *yb, int n, int G0, int lep, int nks,
                        const void *cols, void *Spart, int ntile64, int sms) {
  const size_t smem = yg_umma_sfac_smem(lep);
  if (smem == 0 || nks > UM_KMAX) {
    yg_set_error("tcgen05 Ewald S pass: k-space too large for its shared-memory layout");
    return YG_ERR_UNSUPPORTED;
  }
  int rc;
  if ((rc = yg_smem_optin((const void *)k_sfac_umma, smem))) return rc;
  const int nch = (n + YG_SFAC_ATB - 1) / YG_SFAC_ATB;
  if (nch <= 0) return YG_OK;
  dim3 grid(nch, ntile64);
  k_sfac_umma<<<grid, US_THREADS, smem, ctx->stream>>>((const float2 *)te, (const uint4 *)yb, n, G0, lep, nks,
                                                       (const int4 *)cols, (float2 *)Spart, ntile64, sms,
                                                       ctx->d_status);
  YG_LAUNCH_CHECK(ctx, "k_sfac_umma");
  return YG_OK;
}

// A operand of the atoms [a0, a0 + n) in 128-atom blocks (nblk of them).
int yg_launch_ya_umma(yg_ctx *ctx, const void *yf, int64_t a0, int64_t n, int nmf, int nks, int64_t nblk, void *ya) {
  const int64_t threads = nblk * nks * UM_M * 2;
  if (threads <= 0) return YG_OK;
  k_ya_umma<<<yg_blocks(threads, 256), 256, 0, ctx->stream>>>((const uint2 *)yf, a0, n, nmf, nks, nblk, (uint4 *)ya);
  YG_LAUNCH_CHECK(ctx, "k_ya_umma");
  return YG_OK;
}

// Force pass of atoms [a0, a1) (nab blocks of 128, A operand at ya) over the
// tile ranges urange[0..nr]; writes out[r][atom][3] (r = range).
int yg_launch_force_umma(yg_ctx *ctx, const void *te, const void *ya, int a0, int a1, int ne, int G0, int lep,
                         int nks, const int *urange, int nr, const void *ub, double inv1, double inv2, double *out,
                         int64_t rstride) {
  const size_t smem = yg_umma_force_smem(ne);
  if (smem == 0 || nks > UM_KMAX) {
    yg_set_error("tcgen05 Ewald force pass: k-space too large for its shared-memory layout");
    return YG_ERR_UNSUPPORTED;
  }
  int rc;
  auto kern = k_ewald_force_umma<YG_FORCE_PAIRS != 0>;
  if ((rc = yg_smem_optin((const void *)kern, smem))) return rc;
  const int nab = (a1 - a0 + UM_M - 1) / UM_M;
  if (nab <= 0) return YG_OK;
  dim3 grid(nab, nr);
  kern<<<grid, UM_THREADS, smem, ctx->stream>>>(
      (const float2 *)te, (const uint4 *)ya, a0, a1, ne, G0, lep, nks, ctx->d_ew_upk, ctx->d_ew_upf, urange,
      ctx->d_ew_uoff, (const uint4 *)ub, inv1, inv2, out, rstride, ctx->d_status);
  YG_LAUNCH_CHECK(ctx, "k_ewald_force_umma");
  return YG_OK;
}
