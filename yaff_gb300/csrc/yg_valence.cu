// yg_valence.cu -- kernel (d): the three-layer valence chain.
//
// Forward: relative vectors with the minimum-image wrap (yaff/pes/dlist.c:
// 29-42), internal coordinates (bond, bend cos, bend angle, Urey-Bradley;
// iclist.c:31-55) and harmonic energies (vlist.c:30-34).  Back: dE/dq
// (vlist.c:160-162), the chain rule into relative-vector gradients
// (iclist.c:325-364) and the scatter into gpos and the virial (dlist.c:
// 44-69).  One thread per row of each layer, FP64 throughout; scatters that
// several rows share use FP64 atomics.
#include "yg_internal.cuh"

namespace {

__global__ void k_dlist_fwd(const double *__restrict__ pos, const int2 *__restrict__ ij, int64_t n, CellGeom cell,
                            double *__restrict__ dl) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  int i = ij[r].x, j = ij[r].y;
  double d[3] = {xsub(pos[3 * j], pos[3 * i]), xsub(pos[3 * j + 1], pos[3 * i + 1]),
                 xsub(pos[3 * j + 2], pos[3 * i + 2])};
  int m[3];
  exact_mic(d, cell, m);
  double *o = dl + 6 * r;
  o[0] = d[0]; o[1] = d[1]; o[2] = d[2];
  o[3] = 0.0; o[4] = 0.0; o[5] = 0.0;
}

__device__ __forceinline__ double bend_cos(const double *a, const double *b, double sign) {
  double da = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  double db = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  if (da == 0 || db == 0) return 0.0;
  double dot = a[0] * b[0] + a[1] * b[1] + a[2] * b[2];
  return sign * dot / da / db;
}

__global__ void k_ic_fwd(const int64_t *__restrict__ ic, int64_t n, const double *__restrict__ dl,
                         double *__restrict__ icv, int *__restrict__ bad) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t *row = ic + 9 * r;
  int64_t kind = row[0];
  const double *a = dl + 6 * row[1];
  double v = 0.0;
  if (kind == 0 || kind == 5) {
    v = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  } else if (kind == 1 || kind == 2) {
    const double *b = dl + 6 * row[3];
    v = bend_cos(a, b, (double)(row[2] * row[4]));
    if (kind == 2) {
      if (v > 1.0) v = 1.0;
      if (v < -1.0) v = -1.0;
      v = acos(v);
    }
  } else {
    atomicOr(bad, 1);
  }
  icv[2 * r] = v;
  icv[2 * r + 1] = 0.0;
}

__global__ void k_v_fwd(const double *__restrict__ par, const int *__restrict__ vic, int64_t n,
                        double *__restrict__ icv, double *__restrict__ partial, int want_grad) {
  __shared__ double red[8];
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double e = 0.0;
  if (t < n) {
    double q = icv[2 * vic[t]];
    double x = q - par[2 * t + 1];
    e = 0.5 * par[2 * t] * x * x;
    if (want_grad) atomicAdd(icv + 2 * vic[t] + 1, par[2 * t] * x);
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) e += __shfl_xor_sync(0xffffffffu, e, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = e;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    partial[blockIdx.x] = s;
  }
}

__device__ __forceinline__ void back_bendcos(double *a, double *b, double sign, double value, double grad) {
  double da = sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2]);
  double db = sqrt(b[0] * b[0] + b[1] * b[1] + b[2] * b[2]);
  double ea[3] = {a[0] / da, a[1] / da, a[2] / da};
  double eb[3] = {b[0] / db, b[1] / db, b[2] / db};
  grad *= sign;
  value *= sign;
  double fa = grad / da, fb = grad / db;
  for (int k = 0; k < 3; k++) {
    atomicAdd(a + 3 + k, fa * (eb[k] - value * ea[k]));
    atomicAdd(b + 3 + k, fb * (ea[k] - value * eb[k]));
  }
}

__global__ void k_ic_back(const int64_t *__restrict__ ic, int64_t n, double *__restrict__ dl,
                          const double *__restrict__ icv) {
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (r >= n) return;
  const int64_t *row = ic + 9 * r;
  int64_t kind = row[0];
  double value = icv[2 * r], grad = icv[2 * r + 1];
  double *a = dl + 6 * row[1];
  if (kind == 0 || kind == 5) {
    double x = grad / value;
    for (int k = 0; k < 3; k++) atomicAdd(a + 3 + k, x * a[k]);
  } else if (kind == 1) {
    back_bendcos(a, dl + 6 * row[3], (double)(row[2] * row[4]), value, grad);
  } else if (kind == 2) {
    back_bendcos(a, dl + 6 * row[3], (double)(row[2] * row[4]), cos(value), -grad / sin(value));
  }
}

__global__ void k_dlist_back(const int2 *__restrict__ ij, int64_t n, const double *__restrict__ dl,
                             double *__restrict__ gpos, double *__restrict__ partial) {
  __shared__ double red[8][9];
  int64_t r = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double v[9] = {0, 0, 0, 0, 0, 0, 0, 0, 0};
  if (r < n) {
    const double *o = dl + 6 * r;
    int i = ij[r].x, j = ij[r].y;
    for (int k = 0; k < 3; k++) {
      atomicAdd(gpos + 3 * j + k, o[3 + k]);
      atomicAdd(gpos + 3 * i + k, -o[3 + k]);
    }
    // vtens[3*b + a] += g_a d_b (yaff/pes/dlist.c:59-67)
    for (int b = 0; b < 3; b++)
      for (int a = 0; a < 3; a++) v[3 * b + a] = o[3 + a] * o[b];
  }
  const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
#pragma unroll
  for (int q = 0; q < 9; q++) {
    double x = v[q];
#pragma unroll
    for (int o = 16; o > 0; o >>= 1) x += __shfl_xor_sync(0xffffffffu, x, o);
    v[q] = x;
  }
  if (lane == 0)
    for (int q = 0; q < 9; q++) red[wid][q] = v[q];
  __syncthreads();
  if (threadIdx.x < 9) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w][threadIdx.x];
    partial[(int64_t)blockIdx.x * 9 + threadIdx.x] = s;
  }
}

__global__ void k_store_valence_ev(const double *__restrict__ esum, const double *__restrict__ vsum, int have_v,
                                   double *__restrict__ ev) {
  if (threadIdx.x != 0) return;
  ev[0] = esum[0];
  for (int q = 0; q < 9; q++) ev[1 + q] = have_v ? vsum[q] : 0.0;
}

}  // namespace

int yg_launch_valence(yg_ctx *ctx, int want_grad) {
  const int64_t N = ctx->natom;
  double *gpos = ctx->d_part_gpos + (size_t)YG_PART_VALENCE * N * 3;
  double *ev = ctx->d_part_ev + 10 * YG_PART_VALENCE;
  YG_CUDA(cudaMemsetAsync(gpos, 0, N * 3 * sizeof(double), ctx->stream));
  if (ctx->nterm == 0) {
    YG_CUDA(cudaMemsetAsync(ev, 0, 10 * sizeof(double), ctx->stream));
    ctx->part_valid[YG_PART_VALENCE] = 1;
    return YG_OK;
  }
  int *bad = ctx->d_status + YG_ST_BADCELL;
  YG_CUDA(cudaMemsetAsync(bad, 0, sizeof(int), ctx->stream));
  k_dlist_fwd<<<yg_blocks(ctx->ndelta, 256), 256, 0, ctx->stream>>>(ctx->d_pos, ctx->d_delta_ij, ctx->ndelta,
                                                                    ctx->cell, ctx->d_delta);
  YG_LAUNCH_CHECK(ctx, "k_dlist_fwd");
  k_ic_fwd<<<yg_blocks(ctx->nic, 256), 256, 0, ctx->stream>>>(ctx->d_ic, ctx->nic, ctx->d_delta, ctx->d_icval, bad);
  YG_LAUNCH_CHECK(ctx, "k_ic_fwd");
  const int nbt = yg_blocks(ctx->nterm, 256);
  const int nbd = yg_blocks(ctx->ndelta, 256);
  int rc;
  size_t need = 64 + (size_t)nbt + 1 + (size_t)nbd * 9 + 9;
  if ((rc = yg_ensure(ctx, (void **)&ctx->d_red, &ctx->red_cap, need * sizeof(double)))) return rc;
  double *ep = ctx->d_red + 64;
  double *esum = ep + nbt;
  double *vp = esum + 1;
  double *vsum = vp + (size_t)nbd * 9;
  k_v_fwd<<<nbt, 256, 0, ctx->stream>>>(ctx->d_vpar, ctx->d_vic, ctx->nterm, ctx->d_icval, ep, want_grad);
  YG_LAUNCH_CHECK(ctx, "k_v_fwd");
  if ((rc = yg_launch_reduce_ev(ctx, ep, nbt, 1, esum))) return rc;
  if (want_grad) {
    k_ic_back<<<yg_blocks(ctx->nic, 256), 256, 0, ctx->stream>>>(ctx->d_ic, ctx->nic, ctx->d_delta, ctx->d_icval);
    YG_LAUNCH_CHECK(ctx, "k_ic_back");
    k_dlist_back<<<nbd, 256, 0, ctx->stream>>>(ctx->d_delta_ij, ctx->ndelta, ctx->d_delta, gpos, vp);
    YG_LAUNCH_CHECK(ctx, "k_dlist_back");
    if ((rc = yg_launch_reduce_ev(ctx, vp, nbd, 9, vsum))) return rc;
  }
  k_store_valence_ev<<<1, 32, 0, ctx->stream>>>(esum, vsum, want_grad, ev);
  YG_LAUNCH_CHECK(ctx, "k_store_valence_ev");
  ctx->part_valid[YG_PART_VALENCE] = 1;
  return YG_OK;
}
