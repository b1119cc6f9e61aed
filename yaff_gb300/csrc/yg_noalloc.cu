// yg_noalloc.cu -- Ewald correction without any device allocation.
//
// Some callers cannot let this library allocate device memory: an MD engine
// that owns all device memory through its own pool (a foreign cudaMalloc
// synchronizes the device and fragments that pool), or a step loop that must
// never block on an allocation between steps.  yg_ewald_corr_noalloc serves
// them: the caller passes device buffers for every input and output, and the
// only scratch the computation needs -- the per-block partial sums of the
// energy and virial -- lives in a fixed file-scope device array.
//
// The scratch array is shared by every call in the process (on each device
// that loads the library, which keeps it until exit) and keeps the contents of
// the last call; calls that overlap on the GPU (different streams, or other
// host threads) race on it and must be serialized by the caller.
//
// The scaling table comes from the caller's memory unchecked by the host, so
// the kernel checks every row itself: a row whose indices are not
// 0 <= b < a < natom is skipped (no access through it) and counted in the
// scratch array, and a call that met such a row returns a NaN energy.
#include <atomic>
#include <cstring>

#include "yg_internal.cuh"

#define YG_NOALLOC_BLOCK 256
#define YG_NOALLOC_MAX_BLOCKS (YG_NOALLOC_MAX_ROWS / YG_NOALLOC_BLOCK)
#define YG_NOALLOC_MAX_DEVICES 64

// 4096 blocks x 8 partial sums (energy, 6 virial components and the count of
// rejected rows): 256 KB.
static __device__ __align__(256) double g_noalloc_scratch[YG_NOALLOC_MAX_BLOCKS * 8];

namespace {

// Device address of the scratch array per device, resolved on the first call
// made with that device current.  A cudaDeviceReset ends the context the
// address belongs to; a process that resets a device must not call this entry
// point on that device again.
std::atomic<double *> g_scratch_addr[YG_NOALLOC_MAX_DEVICES];

// One thread per scaling row: the excluded-pair correction of
// yaff/pes/ewald.c:290-335 in FP64, gradients by FP64 atomics, energy and
// virial as fixed-order block partials in the scratch array (slot 7 of a
// block counts its rows with indices outside 0 <= b < a < natom).
__global__ void k_corr_rows(const double *__restrict__ pos, const double *__restrict__ q,
                            const int64_t *__restrict__ sa, const int64_t *__restrict__ sb,
                            const double *__restrict__ scale, int64_t n, int64_t natom, CellGeom cell, double alpha,
                            int64_t nlow, int64_t nhigh, double inv_diel, double *__restrict__ gpos,
                            double *__restrict__ partial) {
  __shared__ double red[YG_NOALLOC_BLOCK / 32][8];
  const int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double vals[8] = {0, 0, 0, 0, 0, 0, 0, 0};
  if (r < n) {
    const int64_t a = sa[r], b = sb[r];
    const bool bad = !(b >= 0 && b < a && a < natom);
    const bool skip = bad || (a < nlow && b < nlow) || (a >= nhigh && b >= nhigh);
    vals[7] = bad ? 1.0 : 0.0;
    if (!skip) {
      double d[3] = {pos[3 * b] - pos[3 * a], pos[3 * b + 1] - pos[3 * a + 1], pos[3 * b + 2] - pos[3 * a + 2]};
      int m[3];
      exact_mic(d, cell, m);
      const double dist = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
      const double x = alpha * dist;
      const double pot = erf(x) / dist;
      const double fac = (1.0 - scale[r]) * q[b] * q[a];
      double g = -fac * (1.1283791670955125739 * alpha * exp(-x * x) - pot) / dist / dist;
      vals[0] = -fac * pot * inv_diel;
      g *= inv_diel;
      if (gpos) {
        for (int k = 0; k < 3; k++) {
          atomicAdd(gpos + 3 * b + k, d[k] * g);
          atomicAdd(gpos + 3 * a + k, -d[k] * g);
        }
      }
      vals[1] = d[0] * d[0] * g;
      vals[2] = d[1] * d[1] * g;
      vals[3] = d[2] * d[2] * g;
      vals[4] = d[1] * d[0] * g;
      vals[5] = d[2] * d[0] * g;
      vals[6] = d[2] * d[1] * g;
    }
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int k = 0; k < 8; k++) {
    double v = vals[k];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    if (lane == 0) red[wid][k] = v;
  }
  __syncthreads();
  if (threadIdx.x < 8) {
    double s = 0.0;
    for (int w = 0; w < YG_NOALLOC_BLOCK / 32; w++) s += red[w][threadIdx.x];
    partial[(int64_t)blockIdx.x * 8 + threadIdx.x] = s;
  }
}

// One block: fixed-order sum of the block partials plus the self term
// -alpha/sqrt(pi) sum q^2 over [nlow, nhigh) (yaff/pes/ewald.c:289-292); a
// call with a rejected scaling row stores a NaN energy.
__global__ void k_corr_finish(const double *__restrict__ partial, int nblocks, const double *__restrict__ q,
                              int64_t nlow, int64_t nhigh, double alpha, double inv_diel, double *__restrict__ energy,
                              double *__restrict__ vtens) {
  __shared__ double sh[9][YG_NOALLOC_BLOCK];
  double acc[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  for (int b = threadIdx.x; b < nblocks; b += blockDim.x)
    for (int k = 0; k < 8; k++) acc[k] += partial[(int64_t)b * 8 + k];
  for (int64_t i = nlow + threadIdx.x; i < nhigh; i += blockDim.x) acc[8] += q[i] * q[i];
  for (int k = 0; k < 9; k++) sh[k][threadIdx.x] = acc[k];
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int k = 0; k < 9; k++) sh[k][threadIdx.x] += sh[k][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double eself = -alpha / 1.7724538509055160273 * sh[8][0];
    if (energy) *energy = sh[7][0] > 0.0 ? __longlong_as_double(0x7ff8000000000000LL) : sh[0][0] + eself * inv_diel;
    if (vtens) {
      const double v[9] = {sh[1][0], sh[4][0], sh[5][0], sh[4][0], sh[2][0], sh[6][0], sh[5][0], sh[6][0], sh[3][0]};
      for (int k = 0; k < 9; k++) vtens[k] = v[k];
    }
  }
}

}  // namespace

extern "C" int yg_ewald_corr_noalloc(const double *pos, const double *charges, int64_t natom,
                                     const int64_t *stab_a, const int64_t *stab_b, const double *stab_scale,
                                     int64_t nstab, const double *rvecs, const double *gvecs, double volume,
                                     double alpha, double dielectric, int64_t nlow, int64_t nhigh, double *energy,
                                     double *gpos, double *vtens, void *stream) {
  if (!pos || !charges || natom <= 0 || !rvecs || !gvecs || !energy || !vtens) {
    yg_set_error("yg_ewald_corr_noalloc: missing argument");
    return YG_ERR_ARG;
  }
  if (nstab < 0 || (nstab > 0 && (!stab_a || !stab_b || !stab_scale))) {
    yg_set_error("yg_ewald_corr_noalloc: bad scaling table");
    return YG_ERR_ARG;
  }
  if (nstab > YG_NOALLOC_MAX_ROWS) {
    yg_set_error("yg_ewald_corr_noalloc: more scaling rows than the fixed scratch holds (max 1048576)");
    return YG_ERR_CAPACITY;
  }
  if (nhigh == -1) nhigh = natom;  // the reference's "up to the last atom" (ff.py _check_nlow_nhigh)
  if (!(alpha > 0.0) || !(dielectric >= 1.0) || nlow < 0 || nhigh < nlow || nhigh > natom) {
    yg_set_error("yg_ewald_corr_noalloc: bad alpha, dielectric or nlow/nhigh");
    return YG_ERR_ARG;
  }
  int dev = 0;
  YG_CUDA(cudaGetDevice(&dev));
  if (dev < 0 || dev >= YG_NOALLOC_MAX_DEVICES) {
    yg_set_error("yg_ewald_corr_noalloc: device index out of range");
    return YG_ERR_ARG;
  }
  // first call on this device: resolve the device address of the scratch
  // array (host code cannot use the symbol itself as a device pointer)
  double *scratch = g_scratch_addr[dev].load(std::memory_order_acquire);
  if (!scratch) {
    void *p = nullptr;
    YG_CUDA(cudaGetSymbolAddress(&p, g_noalloc_scratch));
    scratch = (double *)p;
    // threads racing here all resolve the same address
    g_scratch_addr[dev].store(scratch, std::memory_order_release);
  }
  cudaStream_t st = (cudaStream_t)stream;
  CellGeom cell;
  memcpy(cell.rv, rvecs, 9 * sizeof(double));
  memcpy(cell.gv, gvecs, 9 * sizeof(double));
  cell.volume = volume;
  cell.nvec = 3;
  if (gpos) YG_CUDA(cudaMemsetAsync(gpos, 0, (size_t)natom * 3 * sizeof(double), st));
  const int nb = nstab > 0 ? (int)((nstab + YG_NOALLOC_BLOCK - 1) / YG_NOALLOC_BLOCK) : 0;
  const double inv_diel = 1.0 / dielectric;
  if (nb > 0) {
    k_corr_rows<<<nb, YG_NOALLOC_BLOCK, 0, st>>>(pos, charges, stab_a, stab_b, stab_scale, nstab, natom, cell, alpha,
                                                  nlow, nhigh, inv_diel, gpos, scratch);
    cudaError_t e = cudaGetLastError();
    if (e != cudaSuccess) return yg_cuda_fail(e, "k_corr_rows");
  }
  k_corr_finish<<<1, YG_NOALLOC_BLOCK, 0, st>>>(scratch, nb, charges, nlow, nhigh, alpha, inv_diel, energy, vtens);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return yg_cuda_fail(e, "k_corr_finish");
  return YG_OK;
}
