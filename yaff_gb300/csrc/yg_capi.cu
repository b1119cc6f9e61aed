// yg_capi.cu -- the C ABI of libyaffgb.so (declared in include/yaffgb.h).
//
// Owns the device state of a system (yg_ctx), validates arguments, keeps the
// call-order state machine (cell -> positions -> neighbour list -> parts) and
// turns device-side conditions into status codes.  All kernels are launched on
// the context's stream; the host only blocks where a result must come back
// (neighbour-list capacity check, skin test, result readback).
#include <cmath>
#include <cstdio>
#include <cstring>
#include <map>
#include <mutex>
#include <string>
#include <vector>

#include "yg_internal.cuh"

// The result readback writes the gradient straight into the page-locked
// host mirror through its device alias (1), or sums it in device memory and
// moves it with the copy engine in chunks (0).
#ifndef YG_RB_DIRECT
#define YG_RB_DIRECT 1
#endif
// Where the device can address pageable host memory through the host's page
// tables (cudaDevAttrPageableMemoryAccessUsesHostPageTables, Grace systems),
// the summed gradient is written (or added) into the caller's own array by
// the device after a device-side check of the result status, instead of
// being added by the host from the mirror (1); 0 keeps the mirror path.
#ifndef YG_RB_ATS
#define YG_RB_ATS 1
#endif

namespace {
thread_local std::string g_last_error;
}

void yg_set_error(const std::string &msg) { g_last_error = msg; }

int yg_cuda_fail(cudaError_t err, const char *what) {
  g_last_error = std::string(what) + ": " + cudaGetErrorString(err);
  return YG_ERR_CUDA;
}

namespace {
std::mutex g_pool_mu;
std::map<int, cudaMemPool_t> g_pools;
// pinned host blocks of freed contexts, by power-of-two size class
std::multimap<size_t, void *> g_pinned_free;

// The library's own pool per device: freed memory up to the release
// threshold stays mapped for the next context instead of going back to the
// driver at every synchronization.
int pool_of_current_device(cudaMemPool_t *out) {
  int dev = 0;
  YG_CUDA(cudaGetDevice(&dev));
  std::lock_guard<std::mutex> lk(g_pool_mu);
  auto it = g_pools.find(dev);
  if (it != g_pools.end()) {
    *out = it->second;
    return YG_OK;
  }
  cudaMemPoolProps props;
  memset(&props, 0, sizeof(props));
  props.allocType = cudaMemAllocationTypePinned;
  props.handleTypes = cudaMemHandleTypeNone;
  props.location.type = cudaMemLocationTypeDevice;
  props.location.id = dev;
  cudaMemPool_t pool;
  YG_CUDA(cudaMemPoolCreate(&pool, &props));
  uint64_t keep = (uint64_t)8 << 30;
  YG_CUDA(cudaMemPoolSetAttribute(pool, cudaMemPoolAttrReleaseThreshold, &keep));
  g_pools[dev] = pool;
  *out = pool;
  return YG_OK;
}

size_t pinned_class(size_t bytes) {
  size_t c = 4096;
  while (c < bytes) c <<= 1;
  return c;
}

int pinned_get(size_t bytes, void **out, size_t *cls) {
  *cls = pinned_class(bytes);
  {
    std::lock_guard<std::mutex> lk(g_pool_mu);
    auto it = g_pinned_free.find(*cls);
    if (it != g_pinned_free.end()) {
      *out = it->second;
      g_pinned_free.erase(it);
      return YG_OK;
    }
  }
  YG_CUDA(cudaMallocHost(out, *cls));
  return YG_OK;
}

// Pinned blocks are recycled, never released: cudaFreeHost would synchronize
// the device.
void pinned_put(void *p, size_t cls) {
  if (!p) return;
  std::lock_guard<std::mutex> lk(g_pool_mu);
  g_pinned_free.emplace(cls, p);
}
}  // namespace

int yg_alloc(yg_ctx *ctx, void **ptr, size_t bytes) {
  if (bytes == 0) bytes = 16;
  cudaError_t e = cudaMallocFromPoolAsync(ptr, bytes, ctx->pool, ctx->stream);
  if (e != cudaSuccess) {
    *ptr = nullptr;
    return yg_cuda_fail(e, "cudaMallocFromPoolAsync");
  }
  ctx->alloc_bytes[*ptr] = bytes;
  ctx->alloc_calls++;
  ctx->bytes_now += (int64_t)bytes;
  if (ctx->bytes_now > ctx->bytes_high) ctx->bytes_high = ctx->bytes_now;
  return YG_OK;
}

void yg_free(yg_ctx *ctx, void **ptr) {
  if (*ptr) {
    cudaFreeAsync(*ptr, ctx->stream);
    auto it = ctx->alloc_bytes.find(*ptr);
    if (it != ctx->alloc_bytes.end()) {
      ctx->bytes_now -= (int64_t)it->second;
      ctx->alloc_bytes.erase(it);
    }
  }
  *ptr = nullptr;
}

int yg_ensure(yg_ctx *ctx, void **ptr, size_t *cap, size_t bytes) {
  if (*ptr && *cap >= bytes) return YG_OK;
  yg_free(ctx, ptr);
  size_t want = bytes + bytes / 4 + 256;
  int rc = yg_alloc(ctx, ptr, want);
  if (rc) {
    *cap = 0;
    return rc;
  }
  *cap = want;
  return YG_OK;
}

namespace {
// Sums the requested parts: scalars into out[0..16), the gradient into
// gout[0..3N) (device memory, or the page-locked host mirror through its
// device alias).
__global__ void k_total(const double *__restrict__ part_ev, const double *__restrict__ part_gpos, int64_t natom,
                        int mask, int want_gpos, double *__restrict__ out, double *__restrict__ gout,
                        int *__restrict__ nan_flag) {
  int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < 10) {
    double s = 0.0;
    for (int p = 0; p < YG_NPART; p++)
      if (mask & (1 << p)) s += part_ev[10 * p + t];
    out[t] = s;
  }
  if (t < YG_NPART) out[10 + t] = part_ev[10 * t];
  if (want_gpos && t < natom * 3) {
    double s = 0.0;
    for (int p = 0; p < YG_NPART; p++)
      if (mask & (1 << p)) s += part_gpos[(int64_t)p * natom * 3 + t];
    gout[t] = s;
    if (isnan(s)) atomicOr(nan_flag, 1);
  }
}

// The summed gradient (device memory) into the caller's host array, added
// (add = 1) or written, only when the result is valid: no NaN in the
// gradient or the energy and no bounded wait that gave up.  The caller's
// array is otherwise left as it was.
__global__ void k_total_apply(const double *__restrict__ tot, int64_t n3, int add, const int *__restrict__ status,
                              const double *__restrict__ ev, double *gpos) {
  if (status[YG_ST_NANGRAD] || status[YG_ST_TIMEOUT] || isnan(ev[0])) return;
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n3) gpos[t] = add ? gpos[t] + tot[t] : tot[t];
}

}  // namespace

// Self term of the Ewald correction, -alpha/sqrt(pi) sum q^2 over
// [nlow, nhigh) in the reference's order (yaff/pes/ewald.c:289-292).
double yg_host_self_energy(yg_ctx *ctx) {
  const std::vector<double> &q = ctx->h_charge;
  if (q.empty()) return 0.0;
  double x = ctx->ew_alpha / 1.7724538509055160273;
  double e = 0.0;
  for (int64_t i = ctx->ew_nlow; i < ctx->ew_nhigh; i++) e -= x * q[i] * q[i];
  return e;
}

extern "C" {

const char *yg_status_string(int status) {
  switch (status) {
    case YG_OK: return "ok";
    case YG_ERR_ARG: return "invalid argument";
    case YG_ERR_CUDA: return "CUDA error";
    case YG_ERR_NAN: return "not-a-number in the result";
    case YG_ERR_UNSUPPORTED: return "unsupported";
    case YG_ERR_CAPACITY: return "buffer capacity exceeded";
    case YG_ERR_DENSITY: return "atom density too high";
    case YG_ERR_STATE: return "call order violated";
    default: return "unknown status";
  }
}

const char *yg_last_error(void) { return g_last_error.c_str(); }

int yg_create(int64_t natom, int precision, void *stream, yg_ctx **out) {
  if (!out || natom <= 0 || natom > (int64_t)1 << 30) {
    yg_set_error("natom must be in [1, 2^30]");
    return YG_ERR_ARG;
  }
  if (precision < YG_FP64 || precision > YG_MIXED_KAHAN) {
    yg_set_error("unknown precision mode");
    return YG_ERR_ARG;
  }
  yg_ctx *c = new yg_ctx();
  c->natom = natom;
  c->precision = precision;
  c->stream = (cudaStream_t)stream;
  const size_t N = (size_t)natom;
  int rc = pool_of_current_device(&c->pool);
  if (rc) {
    delete c;
    return rc;
  }
  {
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess ||
        cudaDeviceGetAttribute(&c->nsm, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess || c->nsm < 1)
      c->nsm = 1;
  }
  rc |= yg_alloc(c, (void **)&c->d_pos, N * 3 * sizeof(double));
  rc |= yg_alloc(c, (void **)&c->d_pos_build, N * 3 * sizeof(double));
  rc |= yg_alloc(c, (void **)&c->d_charge, N * sizeof(double));
  rc |= yg_alloc(c, (void **)&c->d_cell_of, N * sizeof(int));
  rc |= yg_alloc(c, (void **)&c->d_wimg, N * 3 * sizeof(int));
  rc |= yg_alloc(c, (void **)&c->d_sorted, N * sizeof(int));
  rc |= yg_alloc(c, (void **)&c->d_rank, N * sizeof(int));
  rc |= yg_alloc(c, (void **)&c->d_org, N * 3 * sizeof(double));
  rc |= yg_alloc(c, (void **)&c->d_x64, N * sizeof(double4_32a));
  rc |= yg_alloc(c, (void **)&c->d_x32, N * sizeof(float4));
  rc |= yg_alloc(c, (void **)&c->d_xb, N * sizeof(float4));
  rc |= yg_alloc(c, (void **)&c->d_ncount, N * sizeof(int2));
  rc |= yg_alloc(c, (void **)&c->d_status, YG_ST_NWORDS * sizeof(int));
  rc |= yg_alloc(c, (void **)&c->d_part_ev, YG_NPART * 10 * sizeof(double));
  rc |= yg_alloc(c, (void **)&c->d_part_gpos, (size_t)YG_NPART * N * 3 * sizeof(double));
  rc |= yg_alloc(c, (void **)&c->d_total, (16 + N * 3) * sizeof(double));
  if (rc == YG_OK) rc = yg_ensure(c, (void **)&c->d_red, &c->red_cap, 4096 * sizeof(double));
  if (rc == YG_OK) {
    // [h_total | 8 u64 words | status words]
    const size_t tot = (16 + N * 3) * sizeof(double);
    if (pinned_get(tot + 64 + YG_ST_NWORDS * sizeof(int), &c->h_block, &c->h_block_bytes) != YG_OK) {
      rc = YG_ERR_CUDA;
    } else {
      c->h_total = (double *)c->h_block;
      c->h_u64 = (unsigned long long *)((char *)c->h_block + tot);
      c->h_status = (int *)((char *)c->h_block + tot + 64);
    }
  }
  if (rc == YG_OK) {
    cudaError_t e = cudaMemsetAsync(c->d_charge, 0, N * sizeof(double), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_part_ev, 0, YG_NPART * 10 * sizeof(double), c->stream);
    if (e == cudaSuccess) e = cudaMemsetAsync(c->d_part_gpos, 0, (size_t)YG_NPART * N * 3 * sizeof(double), c->stream);
    if (e != cudaSuccess) rc = yg_cuda_fail(e, "cudaMemsetAsync");
  }
  if (rc != YG_OK) {
    yg_destroy(c);
    return rc == YG_ERR_CUDA ? YG_ERR_CUDA : rc;
  }
  *out = c;
  return YG_OK;
}

int yg_destroy(yg_ctx *c) {
  if (!c) return YG_OK;
  yg_ewald_join(c);
  cudaStreamSynchronize(c->stream);
  void **bufs[] = {
      (void **)&c->d_pos, (void **)&c->d_pos_build, (void **)&c->d_charge, (void **)&c->d_cell_of,
      (void **)&c->d_wimg, (void **)&c->d_sorted, (void **)&c->d_rank, (void **)&c->d_cell_start,
      (void **)&c->d_cell_fill, (void **)&c->d_org, (void **)&c->d_x64, (void **)&c->d_x32, (void **)&c->d_xb,
      (void **)&c->d_shift64, (void **)&c->d_shift32, (void **)&c->d_cfrac, (void **)&c->d_rows, (void **)&c->d_nbr, (void **)&c->d_ncount,
      (void **)&c->d_status, (void **)&c->d_excl_start, (void **)&c->d_excl, (void **)&c->d_stab_ab,
      (void **)&c->d_stab_scale, (void **)&c->d_pp_src, (void **)&c->d_pp64, (void **)&c->d_pp32,
      (void **)&c->d_ew_pref, (void **)&c->d_ew_tiles, (void **)&c->d_ew_tab, (void **)&c->d_ew_Spart,
      (void **)&c->d_ew_S, (void **)&c->d_ew_W, (void **)&c->d_ew_wslot, (void **)&c->d_ew_gpart, (void **)&c->d_ew_red,
      (void **)&c->d_ew_fpre, (void **)&c->d_ew_fpiece, (void **)&c->d_ew_woff, (void **)&c->d_ew_crange, (void **)&c->d_ew_te,
      (void **)&c->d_ew_yf, (void **)&c->d_ew_ys, (void **)&c->d_ew_wb, (void **)&c->d_ew_uoff, (void **)&c->d_ew_upk, (void **)&c->d_ew_upf, (void **)&c->d_ew_pcols, (void **)&c->d_ew_uslot,
      (void **)&c->d_ew_urange, (void **)&c->d_ew_ya, (void **)&c->d_ew_ub,
      (void **)&c->d_delta_ij, (void **)&c->d_delta, (void **)&c->d_ic, (void **)&c->d_icval, (void **)&c->d_vpar,
      (void **)&c->d_vkind, (void **)&c->d_vE, (void **)&c->d_part_ev, (void **)&c->d_part_gpos,
      (void **)&c->d_total, (void **)&c->d_red, (void **)&c->d_vel, (void **)&c->d_invm, (void **)&c->d_md_ekpart,
      (void **)&c->d_md_ekin, (void **)&c->d_md_log, (void **)&c->d_md_extra, (void **)&c->d_md_step,
      (void **)&c->d_md_ctrl, (void **)&c->d_md_thermo, (void **)&c->d_snap_pos, (void **)&c->d_snap_vel,
      (void **)&c->d_snap_total, (void **)&c->d_snap_step, (void **)&c->d_snap_thermo};
  if (c->md_graph_exec) cudaGraphExecDestroy(c->md_graph_exec);
  if (c->md_cap_stream) cudaStreamDestroy(c->md_cap_stream);
  if (c->ew_aux) cudaStreamDestroy(c->ew_aux);
  if (c->ew_fork_ev) cudaEventDestroy(c->ew_fork_ev);
  for (int k = 0; k < YG_RB_CHUNKS; k++)
    if (c->rb_ev[k]) cudaEventDestroy(c->rb_ev[k]);
  if (c->ew_join_ev) cudaEventDestroy(c->ew_join_ev);
  if (c->pool) {
    for (void **b : bufs) yg_free(c, b);
    for (int p = 0; p < YG_MAX_POT; p++) {
      yg_free(c, (void **)&c->d_ptab64[p]);
      yg_free(c, (void **)&c->d_ptab32[p]);
    }
    // anything the context allocated that no field above names
    std::vector<void *> left;
    for (auto &kv : c->alloc_bytes) left.push_back(kv.first);
    for (void *p : left) yg_free(c, &p);
  }
  pinned_put(c->h_block, c->h_block_bytes);
  delete c;
  return YG_OK;
}

int yg_set_precision(yg_ctx *c, int precision) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c || precision < YG_FP64 || precision > YG_MIXED_KAHAN) return YG_ERR_ARG;
  c->precision = precision;
  return YG_OK;
}

int yg_set_cell(yg_ctx *c, const double *rvecs, const double *gvecs, int nvec, double volume) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c || !rvecs || !gvecs) return YG_ERR_ARG;
  if (nvec != 3) {
    yg_set_error("the device neighbour list supports 3D periodic cells only (nvec == 3)");
    return YG_ERR_UNSUPPORTED;
  }
  if (!(volume > 0.0) || !std::isfinite(volume)) {
    yg_set_error("cell volume must be positive");
    return YG_ERR_ARG;
  }
  memcpy(c->cell.rv, rvecs, 9 * sizeof(double));
  memcpy(c->cell.gv, gvecs, 9 * sizeof(double));
  c->cell.volume = volume;
  c->cell.nvec = nvec;
  c->have_cell = 1;
  c->have_list = 0;
  c->geom_valid = 0;
  return YG_OK;
}

int yg_set_positions(yg_ctx *c, const double *pos, int on_device) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c || !pos) return YG_ERR_ARG;
  YG_CUDA(cudaMemcpyAsync(c->d_pos, pos, c->natom * 3 * sizeof(double),
                          on_device ? cudaMemcpyDeviceToDevice : cudaMemcpyHostToDevice, c->stream));
  c->have_pos = 1;
  for (int p = 0; p < YG_NPART; p++) c->part_valid[p] = 0;
  if (c->have_list) return yg_launch_prep_positions(c);
  return YG_OK;
}

int yg_set_charges(yg_ctx *c, const double *charges) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c || !charges) return YG_ERR_ARG;
  std::vector<double> &h = c->h_charge;
  h.assign(charges, charges + c->natom);
  c->h_qmax = c->h_qsum = 0.0;
  for (double q : h) {
    c->h_qmax = std::max(c->h_qmax, std::fabs(q));
    c->h_qsum += std::fabs(q);
  }
  YG_CUDA(cudaMemcpyAsync(c->d_charge, h.data(), c->natom * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  c->have_charges = 1;
  if (c->have_list) return yg_launch_prep_positions(c);
  return YG_OK;
}

int yg_set_scalings(yg_ctx *c, const int64_t *a, const int64_t *b, const double *scale, const int64_t *nbond,
                    int64_t n) {
  if (!c || n < 0 || (n > 0 && (!a || !b || !scale || !nbond))) return YG_ERR_ARG;
  const int64_t N = c->natom;
  double tab[5] = {1.0, 1.0, 1.0, 1.0, 1.0};
  int seen[5] = {0, 0, 0, 0, 0};
  std::vector<int64_t> cnt(N + 1, 0);
  for (int64_t r = 0; r < n; r++) {
    if (a[r] < 0 || a[r] >= N || b[r] < 0 || b[r] >= N || a[r] <= b[r] || nbond[r] < 1 || nbond[r] > 4) {
      yg_set_error("scaling rows need 0 <= b < a < natom and 1 <= nbond <= 4");
      return YG_ERR_ARG;
    }
    int k = (int)nbond[r];
    if (seen[k] && tab[k] != scale[r]) {
      yg_set_error("scaling rows with the same nbond must share one scale");
      return YG_ERR_ARG;
    }
    seen[k] = 1;
    tab[k] = scale[r];
    cnt[a[r] + 1]++;
    cnt[b[r] + 1]++;
  }
  for (int64_t i = 0; i < N; i++) cnt[i + 1] += cnt[i];
  std::vector<int> start(N + 1);
  for (int64_t i = 0; i <= N; i++) start[i] = (int)cnt[i];
  std::vector<int2> ex(2 * n > 0 ? 2 * n : 1);
  std::vector<int64_t> fill(cnt.begin(), cnt.end() - 1);
  std::vector<int2> ab(n > 0 ? n : 1);
  std::vector<double> sc(n > 0 ? n : 1);
  for (int64_t r = 0; r < n; r++) {
    ex[fill[a[r]]++] = make_int2((int)b[r], (int)nbond[r]);
    ex[fill[b[r]]++] = make_int2((int)a[r], (int)nbond[r]);
    ab[r] = make_int2((int)a[r], (int)b[r]);
    sc[r] = scale[r];
  }
  yg_free(c, (void **)&c->d_excl_start);
  yg_free(c, (void **)&c->d_excl);
  yg_free(c, (void **)&c->d_stab_ab);
  yg_free(c, (void **)&c->d_stab_scale);
  int rc;
  if ((rc = yg_alloc(c, (void **)&c->d_excl_start, (N + 1) * sizeof(int)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_excl, ex.size() * sizeof(int2)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_stab_ab, ab.size() * sizeof(int2)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_stab_scale, sc.size() * sizeof(double)))) return rc;
  YG_CUDA(cudaMemcpyAsync(c->d_excl_start, start.data(), (N + 1) * sizeof(int), cudaMemcpyHostToDevice, c->stream));
  YG_CUDA(cudaMemcpyAsync(c->d_excl, ex.data(), ex.size() * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
  YG_CUDA(cudaMemcpyAsync(c->d_stab_ab, ab.data(), ab.size() * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
  YG_CUDA(cudaMemcpyAsync(c->d_stab_scale, sc.data(), sc.size() * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  c->nexcl = 2 * n;
  c->nstab = n;
  memcpy(c->scale_tab, tab, sizeof(tab));
  c->have_list = 0;  // scaling codes are baked into the list
  return YG_OK;
}

int yg_set_pair_pot(yg_ctx *c, int slot, int kind, const double *sigma, const double *epsilon,
                    const int32_t *onlypauli, const double *radii, double alpha, double dielectric, double rcut,
                    int tr_kind, double tr_par) {
  if (!c || slot < 0 || slot >= YG_MAX_POT) return YG_ERR_ARG;
  if (kind < YG_POT_LJ || kind > YG_POT_GRIMME || tr_kind < YG_TR_NONE || tr_kind > YG_TR_SWITCH3) return YG_ERR_ARG;
  if (!(rcut > 0.0) || !(dielectric > 0.0)) {
    yg_set_error("rcut and dielectric must be positive");
    return YG_ERR_ARG;
  }
  // Grimme: sigma = r0, epsilon = c6 (both mixed like MM3's, r0 summed, c6 geometric)
  if (kind != YG_POT_EI && (!sigma || !epsilon)) return YG_ERR_ARG;
  if ((kind == YG_POT_MM3 || kind == YG_POT_MM3CAP) && !onlypauli) return YG_ERR_ARG;
  PairPotHost &P = c->pot[slot];
  P = PairPotHost();
  P.active = 1;
  P.kind = kind;
  P.tr_kind = tr_kind;
  P.tr_par = tr_par;
  P.rcut = rcut;
  P.alpha = alpha;
  P.dielectric = dielectric;
  const int64_t N = c->natom;
  if (sigma) P.sigma.assign(sigma, sigma + N);
  if (epsilon) {
    P.sqrteps.resize(N);
    for (int64_t i = 0; i < N; i++) {
      if (epsilon[i] < 0.0) {
        yg_set_error("epsilon must be non-negative");
        return YG_ERR_ARG;
      }
      P.sqrteps[i] = std::sqrt(epsilon[i]);
    }
  }
  if (onlypauli) P.onlypauli.assign(onlypauli, onlypauli + N);
  if (radii) {
    bool any = false;
    for (int64_t i = 0; i < N; i++) any |= (radii[i] != 0.0);
    if (any) {
      P.radius2.resize(N);
      for (int64_t i = 0; i < N; i++) P.radius2[i] = radii[i] * radii[i];
    }
  }
  c->pp_dirty = 1;
  if (c->have_list) return yg_pack_pair_params(c);
  return YG_OK;
}

int yg_set_pair_table(yg_ctx *c, int slot, int kind, int64_t nffatype, const int64_t *ffatype_ids,
                      const double *cross0, const double *cross1, const double *cross2, int64_t power,
                      const double *scales, double rcut, int tr_kind, double tr_par) {
  if (!c || slot < 0 || slot >= YG_MAX_POT) return YG_ERR_ARG;
  if (kind < YG_POT_EXPREP || kind > YG_POT_DISP68BJ || tr_kind < YG_TR_NONE || tr_kind > YG_TR_SWITCH3)
    return YG_ERR_ARG;
  if (!(rcut > 0.0)) {
    yg_set_error("rcut must be positive");
    return YG_ERR_ARG;
  }
  if (nffatype <= 0 || nffatype > 4096 || !ffatype_ids || !cross0 || !cross1) return YG_ERR_ARG;
  if (kind == YG_POT_DISP68BJ && (!cross2 || !scales)) return YG_ERR_ARG;
  if (kind == YG_POT_DAMPDISP && (power < 0 || power > 30)) {
    yg_set_error("DampDisp power must be in [0, 30]");
    return YG_ERR_ARG;
  }
  const int64_t N = c->natom, nt = nffatype;
  PairPotHost &P = c->pot[slot];
  P = PairPotHost();
  P.active = 1;
  P.kind = kind;
  P.tr_kind = tr_kind;
  P.tr_par = tr_par;
  P.rcut = rcut;
  P.ntype = (int)nt;
  P.power = (int)power;
  P.types.resize(N);
  for (int64_t i = 0; i < N; i++) {
    if (ffatype_ids[i] < 0 || ffatype_ids[i] >= nt) {
      yg_set_error("atom type index out of range");
      P = PairPotHost();
      return YG_ERR_ARG;
    }
    P.types[i] = (int32_t)ffatype_ids[i];
  }
  // Per type pair (a, b, c, d):
  //   ExpRep, QMDFFRep: (amp, b, 0, 0); LJCross: (eps, sig, 0, 0);
  //   DampDisp: (cn, b, 0, 0);
  //   Disp68BJDamp: (c6_scale c6, c8_scale c8, R^6, R^8), R = bj_a R_cross + bj_b.
  P.table.assign((size_t)nt * nt * 4, 0.0);
  for (int64_t k = 0; k < nt * nt; k++) {
    double *t = P.table.data() + 4 * k;
    if (kind == YG_POT_DISP68BJ) {
      const double R = scales[2] * cross2[k] + scales[3];
      const double R2 = R * R, R4 = R2 * R2;
      t[0] = scales[0] * cross0[k];
      t[1] = scales[1] * cross1[k];
      t[2] = R4 * R2;
      t[3] = R4 * R4;
    } else {
      t[0] = cross0[k];
      t[1] = cross1[k];
    }
  }
  yg_free(c, (void **)&c->d_ptab64[slot]);
  yg_free(c, (void **)&c->d_ptab32[slot]);
  int rc;
  if ((rc = yg_alloc(c, (void **)&c->d_ptab64[slot], (size_t)nt * nt * sizeof(double4_32a)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_ptab32[slot], (size_t)nt * nt * sizeof(float4)))) return rc;
  std::vector<float> t32(P.table.size());
  for (size_t k = 0; k < t32.size(); k++) t32[k] = (float)P.table[k];
  YG_CUDA(cudaMemcpyAsync(c->d_ptab64[slot], P.table.data(), P.table.size() * sizeof(double), cudaMemcpyHostToDevice,
                          c->stream));
  YG_CUDA(cudaMemcpyAsync(c->d_ptab32[slot], t32.data(), t32.size() * sizeof(float), cudaMemcpyHostToDevice,
                          c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  c->pp_dirty = 1;
  if (c->have_list) return yg_pack_pair_params(c);
  return YG_OK;
}

int yg_clear_pair_pots(yg_ctx *c) {
  if (!c) return YG_ERR_ARG;
  for (int p = 0; p < YG_MAX_POT; p++) c->pot[p] = PairPotHost();
  c->pp_dirty = 1;
  return YG_OK;
}

int yg_ewald_wait(yg_ctx *c) {
  if (!c) return YG_ERR_ARG;
  return yg_ewald_join(c);
}

int yg_ewald_info(yg_ctx *c, int *tensor_path, int64_t *nk) {
  if (!c) return YG_ERR_ARG;
  if (tensor_path) {
    int t = c->have_ewald ? c->ew_mma : 0;
    if (t && c->ew_umma && c->ew_force_path == 0) t = 2;
    *tensor_path = t;
  }
  if (nk) *nk = c->have_ewald ? c->ew_nk : 0;
  return YG_OK;
}

int yg_check_wait_timeout(yg_ctx *c, int64_t polls, int *timed_out) {
  if (!c || polls < 1 || polls > (1LL << 24) || !timed_out) return YG_ERR_ARG;
  int rc;
  if ((rc = yg_ewald_join(c))) return rc;
  YG_CUDA(cudaMemsetAsync(c->d_status, 0, YG_ST_NWORDS * sizeof(int), c->stream));
  if ((rc = yg_launch_check_wait_timeout(c, polls))) return rc;
  YG_CUDA(cudaMemcpyAsync(c->h_status, c->d_status, YG_ST_NWORDS * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  *timed_out = c->h_status[YG_ST_TIMEOUT] ? 1 : 0;
  // the self-check's own timeout must not mark the context's next results
  YG_CUDA(cudaMemsetAsync(c->d_status, 0, YG_ST_NWORDS * sizeof(int), c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  c->h_status[YG_ST_TIMEOUT] = 0;
  return YG_OK;
}

int yg_ewald_force_path(yg_ctx *c, int path) {
  if (!c || path < 0 || path > 1) return YG_ERR_ARG;
  int rc;
  if ((rc = yg_ewald_join(c))) return rc;
  c->ew_force_path = path;
  return YG_OK;
}

int yg_ewald_sfac_path(yg_ctx *c, int path) {
  if (!c || path < 0 || path > 2) return YG_ERR_ARG;
  int rc;
  if ((rc = yg_ewald_join(c))) return rc;
  c->ew_sfac_path = path;
  return YG_OK;
}

int yg_nlist_stats(yg_ctx *c, int64_t *nexact, int64_t *maxrow) {
  if (!c) return YG_ERR_ARG;
  if (nexact) *nexact = c->h_status[YG_ST_EXACT];
  if (maxrow) *maxrow = c->h_status[YG_ST_MAXCOUNT];
  return YG_OK;
}

int yg_nlist_build(yg_ctx *c, double rcut_total, const int64_t *rmax, int64_t nlow, int64_t nhigh,
                   int64_t *nneigh) {
  if (!c || !rmax || !(rcut_total > 0.0)) return YG_ERR_ARG;
  if (!c->have_cell || !c->have_pos) {
    yg_set_error("set the cell and the positions before building the neighbour list");
    return YG_ERR_STATE;
  }
  if (nlow < 0 || nhigh < nlow || nhigh > c->natom) {
    yg_set_error("need 0 <= nlow <= nhigh <= natom");
    return YG_ERR_ARG;
  }
  if (c->natom / c->cell.volume > 10.0) {
    yg_set_error("Atom density too high");
    return YG_ERR_DENSITY;
  }
  for (int k = 0; k < 3; k++) {
    if (rmax[k] < 0 || rmax[k] > 1000) return YG_ERR_ARG;
    c->rmax[k] = rmax[k];
  }
  c->rcut_total = rcut_total;
  c->nlow = nlow;
  c->nhigh = nhigh;
  if (c->build_pending) {  // superseded: its status no longer matters
    YG_CUDA(cudaEventSynchronize(c->build_ev));
    c->build_pending = 0;
  }
  int retry = 0;
  int rc = yg_launch_nlist_build(c, rcut_total * rcut_total, &retry);
  if (rc) {
    c->have_list = 0;
    return rc;
  }
  // a new list invalidates the pair parts only (the Ewald and valence parts
  // do not use it; the reciprocal sum may already have been launched)
  for (int p = 0; p < YG_MAX_POT; p++) c->part_valid[YG_PART_PAIR0 + p] = 0;
  if (nneigh) *nneigh = c->nneigh;
  return YG_OK;
}

int yg_nlist_build_async(yg_ctx *c, double rcut_total, const int64_t *rmax, int64_t nlow, int64_t nhigh) {
  if (!c || !rmax || !(rcut_total > 0.0)) return YG_ERR_ARG;
  if (!c->have_cell || !c->have_pos) {
    yg_set_error("set the cell and the positions before building the neighbour list");
    return YG_ERR_STATE;
  }
  if (nlow < 0 || nhigh < nlow || nhigh > c->natom) {
    yg_set_error("need 0 <= nlow <= nhigh <= natom");
    return YG_ERR_ARG;
  }
  if (c->natom / c->cell.volume > 10.0) {
    yg_set_error("Atom density too high");
    return YG_ERR_DENSITY;
  }
  for (int k = 0; k < 3; k++) {
    if (rmax[k] < 0 || rmax[k] > 1000) return YG_ERR_ARG;
    c->rmax[k] = rmax[k];
  }
  c->rcut_total = rcut_total;
  c->nlow = nlow;
  c->nhigh = nhigh;
  if (c->build_pending) {
    YG_CUDA(cudaEventSynchronize(c->build_ev));
    c->build_pending = 0;
  }
  const int rc = yg_launch_nlist_build_async(c, rcut_total * rcut_total);
  if (rc) {
    c->have_list = 0;
    return rc;
  }
  for (int p = 0; p < YG_MAX_POT; p++) c->part_valid[YG_PART_PAIR0 + p] = 0;
  return YG_OK;
}

int yg_nlist_build_wait(yg_ctx *c, int64_t *nneigh) {
  if (!c) return YG_ERR_ARG;
  const int rc = yg_launch_nlist_build_wait(c);
  if (rc == YG_OK && nneigh) *nneigh = c->nneigh;
  return rc;
}

int yg_nlist_recompute(yg_ctx *c) {
  if (!c) return YG_ERR_ARG;
  if (c->build_pending) {
    const int wrc = yg_launch_nlist_build_wait(c);
    if (wrc) return wrc;
  }
  if (!c->have_list || !c->rows_valid) {
    yg_set_error("no neighbour list to recompute");
    return YG_ERR_STATE;
  }
  c->list_recomputed = 1;
  return yg_launch_prep_positions(c);
}

int yg_nlist_max_disp2(yg_ctx *c, double *out) {
  if (!c || !out) return YG_ERR_ARG;
  if (!c->have_list || !c->rows_valid) {
    *out = INFINITY;
    return YG_OK;
  }
  return yg_launch_max_disp2(c, out);
}

int yg_nlist_export(yg_ctx *c, yg_neigh_row *rows, int64_t cap, int64_t *n) {
  if (!c || !n) return YG_ERR_ARG;
  if (c->build_pending) {
    const int wrc = yg_launch_nlist_build_wait(c);
    if (wrc) return wrc;
  }
  if (!c->have_list || !c->rows_valid) {
    yg_set_error("no neighbour list");
    return YG_ERR_STATE;
  }
  return yg_launch_nlist_export(c, rows, cap, n);
}

int yg_pair_compute(yg_ctx *c, int slot_mask, int want_grad) {
  if (!c) return YG_ERR_ARG;
  if (!c->have_list || !c->rows_valid) {
    yg_set_error("build the neighbour list first");
    return YG_ERR_STATE;
  }
  for (int p = 0; p < YG_MAX_POT; p++)
    if ((slot_mask & (1 << p)) && c->pot[p].active && c->pot[p].rcut > c->rcut_total) {
      yg_set_error("pair potential cutoff exceeds the neighbour-list cutoff");
      return YG_ERR_ARG;
    }
  if (c->pp_dirty) {
    int rc = yg_pack_pair_params(c);
    if (rc) return rc;
  }
  return yg_launch_pair(c, slot_mask, want_grad);
}

int yg_ewald_setup(yg_ctx *c, double alpha, double gcut, const int64_t *gmax, double dielectric, int64_t nlow,
                   int64_t nhigh) {
  if (!c || !gmax || !(alpha > 0.0) || !(gcut > 0.0) || !(dielectric >= 1.0)) return YG_ERR_ARG;
  if (!c->have_cell) return YG_ERR_STATE;
  if (nlow < 0 || nhigh < nlow || nhigh > c->natom) return YG_ERR_ARG;
  for (int k = 0; k < 3; k++) {
    if (gmax[k] < 0 || gmax[k] > 4096) return YG_ERR_ARG;
    c->ew_gmax[k] = gmax[k];
  }
  c->ew_alpha = alpha;
  c->ew_gcut = gcut;
  c->ew_diel = dielectric;
  c->ew_nlow = nlow;
  c->ew_nhigh = nhigh;
  return yg_launch_ewald_setup(c);
}

int yg_ewald_reci(yg_ctx *c, int want_grad) {
  if (!c) return YG_ERR_ARG;
  if (!c->have_ewald || !c->have_pos || !c->have_charges) {
    yg_set_error("Ewald needs yg_ewald_setup, positions and charges");
    return YG_ERR_STATE;
  }
  return yg_launch_ewald_reci(c, want_grad);
}

int yg_ewald_corr(yg_ctx *c, int want_grad) {
  if (!c) return YG_ERR_ARG;
  if (!c->have_ewald || !c->have_pos || !c->have_charges) {
    yg_set_error("Ewald needs yg_ewald_setup, positions and charges");
    return YG_ERR_STATE;
  }
  if (c->nstab > 0 && !c->d_stab_ab) return YG_ERR_STATE;
  return yg_launch_ewald_corr(c, want_grad);
}

int yg_set_valence(yg_ctx *c, const int64_t *delta_ij, int64_t ndelta, const int64_t *ic_rows, int64_t nic,
                   const int64_t *vterm_kind, const double *vterm_pars, const int64_t *vterm_ic, int64_t nterm) {
  if (!c || ndelta < 0 || nic < 0 || nterm < 0) return YG_ERR_ARG;
  if ((ndelta && !delta_ij) || (nic && !ic_rows) || (nterm && (!vterm_kind || !vterm_pars || !vterm_ic)))
    return YG_ERR_ARG;
  const int64_t N = c->natom;
  std::vector<int2> ij(ndelta > 0 ? ndelta : 1);
  for (int64_t r = 0; r < ndelta; r++) {
    int64_t i = delta_ij[2 * r], j = delta_ij[2 * r + 1];
    if (i < 0 || i >= N || j < 0 || j >= N || i == j) return YG_ERR_ARG;
    ij[r] = make_int2((int)i, (int)j);
  }
  for (int64_t r = 0; r < nic; r++) {
    const int64_t kind = ic_rows[9 * r];
    if (kind < 0 || kind > 17) {
      yg_set_error("unknown internal-coordinate kind (0..17)");
      return YG_ERR_UNSUPPORTED;
    }
    // relative vectors a kind reads (yaff/pes/iclist.py:231-530)
    const int nused = (kind == 0 || kind == 5) ? 1 : (kind == 1 || kind == 2) ? 2 : 3;
    for (int u = 0; u < nused; u++) {
      const int64_t d = ic_rows[9 * r + 1 + 2 * u], sg = ic_rows[9 * r + 2 + 2 * u];
      if (d < 0 || d >= ndelta || (sg != 1 && sg != -1)) return YG_ERR_ARG;
    }
  }
  std::vector<int4> vk(nterm > 0 ? nterm : 1);
  for (int64_t t = 0; t < nterm; t++) {
    const int64_t kind = vterm_kind[t], i0 = vterm_ic[2 * t], i1 = vterm_ic[2 * t + 1];
    if (kind < 0 || kind > 15) {
      yg_set_error("unknown valence-term kind (0..15)");
      return YG_ERR_UNSUPPORTED;
    }
    if (i0 < 0 || i0 >= nic) return YG_ERR_ARG;
    if (kind == 3 ? (i1 < 0 || i1 >= nic) : (i1 != -1)) return YG_ERR_ARG;
    vk[t] = make_int4((int)kind, (int)i0, (int)i1, 0);
  }
  void **bufs[] = {(void **)&c->d_delta_ij, (void **)&c->d_delta, (void **)&c->d_ic, (void **)&c->d_icval,
                   (void **)&c->d_vpar,     (void **)&c->d_vkind, (void **)&c->d_vE};
  for (void **b : bufs) yg_free(c, b);
  int rc;
  if ((rc = yg_alloc(c, (void **)&c->d_delta_ij, ij.size() * sizeof(int2)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_delta, (size_t)(ndelta > 0 ? ndelta : 1) * 6 * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_ic, (size_t)(nic > 0 ? nic : 1) * 9 * sizeof(int64_t)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_icval, (size_t)(nic > 0 ? nic : 1) * 2 * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_vpar, (size_t)(nterm > 0 ? nterm : 1) * 6 * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_vkind, vk.size() * sizeof(int4)))) return rc;
  YG_CUDA(cudaMemcpyAsync(c->d_delta_ij, ij.data(), ij.size() * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
  if (nic > 0)
    YG_CUDA(cudaMemcpyAsync(c->d_ic, ic_rows, (size_t)nic * 9 * sizeof(int64_t), cudaMemcpyHostToDevice, c->stream));
  if (nterm > 0)
    YG_CUDA(cudaMemcpyAsync(c->d_vpar, vterm_pars, (size_t)nterm * 6 * sizeof(double), cudaMemcpyHostToDevice,
                            c->stream));
  YG_CUDA(cudaMemcpyAsync(c->d_vkind, vk.data(), vk.size() * sizeof(int4), cudaMemcpyHostToDevice, c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  c->ndelta = ndelta;
  c->nic = nic;
  c->nterm = nterm;
  return YG_OK;
}

int yg_valence_compute(yg_ctx *c, int want_grad) {
  if (!c) return YG_ERR_ARG;
  if (!c->have_pos || !c->have_cell) return YG_ERR_STATE;
  return yg_launch_valence(c, want_grad);
}

int yg_get_part(yg_ctx *c, int part, double *energy, double *gpos, double *vtens) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c || part < 0 || part >= YG_NPART) return YG_ERR_ARG;
  if (c->build_pending) {
    const int wrc = yg_launch_nlist_build_wait(c);
    if (wrc) {
      for (int p = 0; p < YG_MAX_POT; p++) c->part_valid[YG_PART_PAIR0 + p] = 0;
      return wrc;
    }
  }
  if (!c->part_valid[part]) {
    yg_set_error("part has no valid result for the current positions");
    return YG_ERR_STATE;
  }
  double ev[10];
  YG_CUDA(cudaMemcpyAsync(ev, c->d_part_ev + 10 * part, sizeof(ev), cudaMemcpyDeviceToHost, c->stream));
  if (gpos)
    YG_CUDA(cudaMemcpyAsync(gpos, c->d_part_gpos + (size_t)part * c->natom * 3, c->natom * 3 * sizeof(double),
                            cudaMemcpyDeviceToHost, c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  if (energy) *energy = ev[0];
  if (vtens) memcpy(vtens, ev + 1, 9 * sizeof(double));
  if (std::isnan(ev[0])) return YG_ERR_NAN;
  return YG_OK;
}

static int get_total(yg_ctx *c, int part_mask, double *energy, double *gpos, double *vtens, double *part_energies,
                     int add);

int yg_get_total(yg_ctx *c, int part_mask, double *energy, double *gpos, double *vtens, double *part_energies) {
  return get_total(c, part_mask, energy, gpos, vtens, part_energies, 0);
}

int yg_get_total_add(yg_ctx *c, int part_mask, double *energy, double *gpos, double *vtens,
                     double *part_energies) {
  return get_total(c, part_mask, energy, gpos, vtens, part_energies, 1);
}

// The summed parts: written into (add = 0) or added to (add = 1) the
// caller's gpos / vtens, straight from the page-locked readback block.
static int get_total(yg_ctx *c, int part_mask, double *energy, double *gpos, double *vtens, double *part_energies,
                     int add) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c) return YG_ERR_ARG;
  if (c->build_pending) {  // the rows of an enqueued build fed the pair parts
    const int wrc = yg_launch_nlist_build_wait(c);
    if (wrc) {
      for (int p = 0; p < YG_MAX_POT; p++) c->part_valid[YG_PART_PAIR0 + p] = 0;
      return wrc;
    }
  }
  for (int p = 0; p < YG_NPART; p++)
    if ((part_mask & (1 << p)) && !c->part_valid[p]) {
      yg_set_error("a requested part has no valid result");
      return YG_ERR_STATE;
    }
  const int64_t n3 = c->natom * 3;
  const int want_gpos = gpos != nullptr;
  int64_t nthreads = want_gpos ? std::max<int64_t>(n3, 16) : 16;
  YG_CUDA(cudaMemsetAsync(c->d_status + YG_ST_NANGRAD, 0, sizeof(int), c->stream));
  // the gradient goes into the caller's array from the device when it can
  // address pageable host memory, else straight into the page-locked mirror
  // when the device can address that (both checked once per context), so no
  // separate copy follows
  if (c->ats_state == 0) {
    int dev = 0, v = 0;
    c->ats_state = -1;
#if YG_RB_ATS
    if (cudaGetDevice(&dev) == cudaSuccess &&
        cudaDeviceGetAttribute(&v, cudaDevAttrPageableMemoryAccessUsesHostPageTables, dev) == cudaSuccess && v == 1)
      c->ats_state = 1;
#endif
    cudaGetLastError();
  }
  const bool ats = want_gpos && c->ats_state == 1;
  if (c->h_total_dev_state == 0) {
    void *alias = nullptr;
#if YG_RB_DIRECT
    const cudaError_t ae = cudaHostGetDevicePointer(&alias, c->h_total, 0);
#else
    const cudaError_t ae = cudaErrorNotSupported;  // always the copy-engine path
#endif
    c->h_total_dev = (ae == cudaSuccess) ? (double *)alias : nullptr;
    c->h_total_dev_state = 1;
    if (ae != cudaSuccess) cudaGetLastError();  // clear the error of the query
  }
  double *gout = (want_gpos && c->h_total_dev && !ats) ? c->h_total_dev + 16 : c->d_total + 16;
  k_total<<<yg_blocks(nthreads, 256), 256, 0, c->stream>>>(c->d_part_ev, c->d_part_gpos, c->natom, part_mask,
                                                          want_gpos, c->d_total, gout, c->d_status + YG_ST_NANGRAD);
  YG_LAUNCH_CHECK(c, "k_total");
  if (ats) {
    k_total_apply<<<yg_blocks(n3, 256), 256, 0, c->stream>>>(c->d_total + 16, n3, add, c->d_status, c->d_total, gpos);
    YG_LAUNCH_CHECK(c, "k_total_apply");
  }
  // status and scalars first, then the gradient in chunks: the host adds
  // (or copies) chunk k while chunk k + 1 is still being transferred
  YG_CUDA(cudaMemcpyAsync(c->h_status, c->d_status, YG_ST_NWORDS * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
  YG_CUDA(cudaMemcpyAsync(c->h_total, c->d_total, 16 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  const bool direct = want_gpos && c->h_total_dev && !ats;
  const int nchunk = (!want_gpos || direct || ats) ? 0 : (n3 >= (1 << 16) ? YG_RB_CHUNKS : 1);
  int64_t cut[YG_RB_CHUNKS + 1];
  for (int k = 0; k <= nchunk; k++) cut[k] = n3 * k / (nchunk ? nchunk : 1);
  for (int k = 0; k < nchunk; k++) {
    if (!c->rb_ev[k]) YG_CUDA(cudaEventCreateWithFlags(&c->rb_ev[k], cudaEventDisableTiming));
    YG_CUDA(cudaMemcpyAsync(c->h_total + 16 + cut[k], c->d_total + 16 + cut[k], (cut[k + 1] - cut[k]) * sizeof(double),
                            cudaMemcpyDeviceToHost, c->stream));
    YG_CUDA(cudaEventRecord(c->rb_ev[k], c->stream));
  }
  if (nchunk) YG_CUDA(cudaEventSynchronize(c->rb_ev[0]));
  else YG_CUDA(cudaStreamSynchronize(c->stream));
  int rc = YG_OK;
  if (c->h_status[YG_ST_TIMEOUT]) {
    yg_set_error("a bounded wait on an asynchronous copy gave up; results are invalid");
    rc = YG_ERR_CUDA;
  } else if (std::isnan(c->h_total[0])) {
    rc = YG_ERR_NAN;
  } else if (want_gpos && c->h_status[YG_ST_NANGRAD]) {
    yg_set_error("not-a-number in the gradient");
    rc = YG_ERR_NAN;
  }
  if (rc == YG_OK || rc == YG_ERR_NAN) {
    if (energy) *energy = c->h_total[0];
    if (part_energies) memcpy(part_energies, c->h_total + 10, YG_NPART * sizeof(double));
  }
  if (rc) {
    YG_CUDA(cudaStreamSynchronize(c->stream));  // no copy left in flight into the mirror
    return rc;
  }
  if (vtens) {
    if (add)
      for (int k = 0; k < 9; k++) vtens[k] += c->h_total[1 + k];
    else
      memcpy(vtens, c->h_total + 1, 9 * sizeof(double));
  }
  if (ats) return YG_OK;  // the device has added (or written) the gradient
  if (direct) {
    cut[0] = 0;
    cut[1] = n3;
  }
  for (int k = 0; k < (direct ? 1 : nchunk); k++) {
    if (k) YG_CUDA(cudaEventSynchronize(c->rb_ev[k]));
    const double *src = c->h_total + 16 + cut[k];
    double *dst = gpos + cut[k];
    const int64_t m = cut[k + 1] - cut[k];
    if (add)
      for (int64_t q = 0; q < m; q++) dst[q] += src[q];
    else
      memcpy(dst, src, m * sizeof(double));
  }
  return YG_OK;
}

int yg_sync(yg_ctx *c) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c) return YG_ERR_ARG;
  YG_CUDA(cudaStreamSynchronize(c->stream));
  return YG_OK;
}

int64_t yg_launch_count(yg_ctx *c) { return c ? c->launches : -1; }

int yg_mem_usage(yg_ctx *c, int64_t *bytes_now, int64_t *bytes_high) {
  if (!c) return YG_ERR_ARG;
  if (bytes_now) *bytes_now = c->bytes_now;
  if (bytes_high) *bytes_high = c->bytes_high;
  return YG_OK;
}

int yg_pool_usage(int64_t *used_now, int64_t *used_high, int64_t *reserved) {
  cudaMemPool_t pool;
  int rc = pool_of_current_device(&pool);
  if (rc) return rc;
  uint64_t v = 0;
  if (used_now) {
    YG_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemCurrent, &v));
    *used_now = (int64_t)v;
  }
  if (used_high) {
    YG_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrUsedMemHigh, &v));
    *used_high = (int64_t)v;
  }
  if (reserved) {
    YG_CUDA(cudaMemPoolGetAttribute(pool, cudaMemPoolAttrReservedMemCurrent, &v));
    *reserved = (int64_t)v;
  }
  return YG_OK;
}

}  // extern "C"
