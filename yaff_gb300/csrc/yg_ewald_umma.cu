// yg_ewald_umma.cu -- force pass of the mixed-precision reciprocal sum on the
// fifth-generation tensor cores (tcgen05.mma, accumulators in tensor memory).
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
// stride (8-row) byte offset 256, descriptor version 1, no swizzle
__device__ __forceinline__ uint64_t um_desc(unsigned saddr) {
  return (uint64_t)((saddr >> 4) & 0x3FFFu) | ((uint64_t)(128 >> 4) << 16) | ((uint64_t)(256 >> 4) << 32) |
         ((uint64_t)1 << 46);
}

__device__ __forceinline__ void um_mma(unsigned dtmem, uint64_t adesc, uint64_t bdesc, unsigned accumulate) {
  asm volatile(
      "{\n.reg .pred p;\nsetp.ne.b32 p, %4, 0;\n"
      "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n}" ::"r"(dtmem),
      "l"(adesc), "l"(bdesc), "r"(UM_IDESC), "r"(accumulate)
      : "memory");
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

__global__ void __launch_bounds__(UM_THREADS, 1)
    k_ewald_force_umma(const float2 *__restrict__ te, const uint4 *__restrict__ ya, int a0, int a1, int ne, int G0,
                       int lep, int nks, const int *__restrict__ upk, const int *__restrict__ urange,
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
#pragma unroll 1
      for (int c = h; c < UM_N / 32; c += HQ) {
        const int4 ca = na, cb = nb;
        const bool last = c + HQ >= UM_N / 32 || ca.x < 0;  // (padding: the rest of the tile is padding)
        if (!last || i + 1 < ntile) {
          const int4 *p = reinterpret_cast<const int4 *>(
              upk + (size_t)(u0 + (last ? i + 1 : i)) * UM_COLS + 8 * (last ? h : c + HQ));
          na = __ldg(p);
          nb = __ldg(p + 1);
        }
        if (ca.x < 0) break;
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
            p0 += (float)(n0 ? -ag0 : ag0) * im1;
            p1 += (float)(n1 ? G0 + 1 - ag1 : ag1 - G0 - 1) * im1;
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

}  // namespace

// Dynamic shared memory of the tcgen05 force pass for ne E0|E1 entries per
// atom; 0 when it does not fit on a multiprocessor.
size_t yg_umma_force_smem(int ne) {
  const size_t need = UM_SMEM_A + 2 * UM_SMEM_B + (size_t)ne * UM_M * sizeof(float2);
  return need <= 225 * 1024 ? need : 0;
}

int yg_umma_kmax() { return UM_KMAX; }
int yg_umma_cols() { return UM_COLS; }

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
  if ((rc = yg_smem_optin((const void *)k_ewald_force_umma, smem))) return rc;
  const int nab = (a1 - a0 + UM_M - 1) / UM_M;
  if (nab <= 0) return YG_OK;
  dim3 grid(nab, nr);
  k_ewald_force_umma<<<grid, UM_THREADS, smem, ctx->stream>>>(
      (const float2 *)te, (const uint4 *)ya, a0, a1, ne, G0, lep, nks, ctx->d_ew_upk, urange,
      ctx->d_ew_uoff, (const uint4 *)ub, inv1, inv2, out, rstride, ctx->d_status);
  YG_LAUNCH_CHECK(ctx, "k_ewald_force_umma");
  return YG_OK;
}
