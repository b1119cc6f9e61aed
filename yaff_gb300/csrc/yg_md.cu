// yg_md.cu -- device-resident velocity Verlet driven entirely by the GPU.
//
// The integration step of yaff/sampling/verlet.py:339-367 (half kick, drift,
// force evaluation, half kick) with positions, velocities, masses and the
// neighbour list resident in HBM.  The reference's skin test
// (yaff/pes/nlist.py:207-218: rebuild when 2 (rmax+1) max|r - r_build| >=
// skin) is evaluated on the device and gates the rebuild kernels, so a whole
// step -- drift, skin test, conditional rebuild, cell-local coordinates,
// fused pair terms, Ewald, valence, device-side sum of the parts, second
// kick, energy log -- is one sequence with no host synchronization.  It is
// captured once into a CUDA graph and replayed; the host reads the status
// words once per batch of steps.  A neighbour row that overflowed its slot
// during a device rebuild is detected at the end of the batch: the batch is
// rolled back to its snapshot, the slots grow, and the batch runs again.
#include <cmath>
#include <cstring>
#include <vector>

#include "yg_internal.cuh"

#define YG_MD_BATCH 128   // steps between host status checks

namespace {

// vel += 0.5 dt a; pos += dt vel   (a = -gpos / m, gpos from the last total)
__global__ void k_kick_drift(double *__restrict__ pos, double *__restrict__ vel, const double *__restrict__ gpos,
                             const double *__restrict__ invm, int64_t natom, double dt) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t >= natom * 3) return;
  const double a = -gpos[t] * invm[t / 3];
  const double v = vel[t] + 0.5 * a * dt;
  vel[t] = v;
  pos[t] += dt * v;
}

// vel += 0.5 dt a; per-block partial kinetic energy
__global__ void k_kick(double *__restrict__ vel, const double *__restrict__ gpos, const double *__restrict__ invm,
                       int64_t natom, double dt, double *__restrict__ ekin_part) {
  __shared__ double red[8];
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double ek = 0.0;
  if (t < natom * 3) {
    const double im = invm[t / 3];
    const double v = vel[t] + 0.5 * (-gpos[t] * im) * dt;
    vel[t] = v;
    ek = 0.5 * v * v / im;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ek += __shfl_xor_sync(0xffffffffu, ek, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ek;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    ekin_part[blockIdx.x] = s;
  }
}

// log[step] = (epot, ekin) from the device-side totals; step++
__global__ void k_md_log(const double *__restrict__ total, const double *__restrict__ ekin, const double *__restrict__ extra,
                         double *__restrict__ log, int *__restrict__ step, int64_t max_rows) {
  if (threadIdx.x != 0) return;
  const int s = *step;
  if (s < max_rows) {
    log[2 * s] = total[0] + *extra;
    log[2 * s + 1] = *ekin;
  }
  *step = s + 1;
}

__global__ void k_total_dev(const double *__restrict__ part_ev, const double *__restrict__ part_gpos, int64_t natom,
                            int mask, double *__restrict__ out) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < 10) {
    double s = 0.0;
    for (int p = 0; p < YG_NPART; p++)
      if (mask & (1 << p)) s += part_ev[10 * p + t];
    out[t] = s;
  }
  if (t < natom * 3) {
    double s = 0.0;
    for (int p = 0; p < YG_NPART; p++)
      if (mask & (1 << p)) s += part_gpos[(int64_t)p * natom * 3 + t];
    out[16 + t] = s;
  }
}

// The skin test of the step: gate = force || !(sqrt(d2) * factor < skin)
// (also set for NaN); clears the displacement word for the next step.
__global__ void k_skin_gate(int *__restrict__ ctrl, double factor, double skin) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  unsigned long long *d2w = (unsigned long long *)(ctrl + 6);
  const double d2 = __longlong_as_double((long long)*d2w);
  *d2w = 0ull;
  const double disp = sqrt(d2) * factor;
  const int gate = ctrl[1] || !(disp < skin);
  ctrl[0] = gate;
  if (gate) {
    ctrl[1] = 0;
    ctrl[2] += 1;
  }
}

__global__ void k_set_int(int *__restrict__ p, int v) {
  if (threadIdx.x == 0 && blockIdx.x == 0) *p = v;
}

// --- thermostats (yaff/sampling/nvt.py:110-500) ---

// Counter-based generator Philox4x32-10 (Salmon, Moraes, Dror, Shaw, "Parallel
// random numbers: as easy as 1, 2, 3", SC'11): ten rounds of two 32x32->64
// multiplications with the round keys bumped by the Weyl constants.
__device__ __forceinline__ uint4 philox4x32(uint4 c, uint2 k) {
#pragma unroll
  for (int r = 0; r < 10; r++) {
    const unsigned lo0 = 0xD2511F53u * c.x, hi0 = __umulhi(0xD2511F53u, c.x);
    const unsigned lo1 = 0xCD9E8D57u * c.z, hi1 = __umulhi(0xCD9E8D57u, c.z);
    c = make_uint4(hi1 ^ c.y ^ k.x, lo1, hi0 ^ c.w ^ k.y, lo0);
    k.x += 0x9E3779B9u;
    k.y += 0xBB67AE85u;
  }
  return c;
}

// A standard normal number for (index, step, stage) of stream `seed`
// (Box-Muller on two 32-bit uniforms in (0, 1)).
__device__ __forceinline__ double normal01(unsigned long long seed, unsigned long long index, int step, int stage) {
  const uint4 r = philox4x32(make_uint4((unsigned)index, (unsigned)(index >> 32), (unsigned)step, (unsigned)stage),
                             make_uint2((unsigned)seed, (unsigned)(seed >> 32)));
  const double u1 = ((double)r.x + 0.5) * 2.3283064365386963e-10;
  const double u2 = ((double)r.y + 0.5) * 2.3283064365386963e-10;
  return sqrt(-2.0 * log(u1)) * cospi(2.0 * u2);
}

// vel *= f[1]
__global__ void k_scale_vel(double *__restrict__ vel, int64_t n3, const double *__restrict__ f) {
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (t < n3) vel[t] *= f[1];
}

// Berendsen: c = sqrt(1 + dt/tau (T0/T - 1)) from the current kinetic energy
// (nvt.py:150-156).
__global__ void k_berendsen(double *__restrict__ th, double *__restrict__ ekin, double kT, double dt_tau, double ndof) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double ek = *ekin;
  const double c = sqrt(1.0 + dt_tau * (kT * ndof / (2.0 * ek) - 1.0));
  th[1] = c;
  th[0] += (1.0 - c * c) * ek;
  *ekin = c * c * ek;
}

// Langevin half step v = c1 v + sqrt((1 - c1^2) kT / m) xi (nvt.py:208-213),
// with per-block partial kinetic energies of the new velocities.
__global__ void k_langevin(double *__restrict__ vel, const double *__restrict__ invm, int64_t natom, double c1,
                           double kT, unsigned long long seed, const int *__restrict__ step, int stage,
                           double *__restrict__ ekin_part) {
  __shared__ double red[8];
  const int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  double ek = 0.0;
  if (t < natom * 3) {
    const double im = invm[t / 3];
    const double v = c1 * vel[t] + sqrt((1.0 - c1 * c1) * kT * im) * normal01(seed, (unsigned long long)t, *step, stage);
    vel[t] = v;
    ek = 0.5 * v * v / im;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) ek += __shfl_xor_sync(0xffffffffu, ek, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = ek;
  __syncthreads();
  if (threadIdx.x == 0) {
    double s = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) s += red[w];
    ekin_part[blockIdx.x] = s;
  }
}

__global__ void k_save_ekin(double *__restrict__ th, const double *__restrict__ ekin) {
  if (threadIdx.x == 0 && blockIdx.x == 0) th[2] = *ekin;
}

// conserved-energy correction of a stochastic update: ekin before - after
__global__ void k_ekin_delta(double *__restrict__ th, const double *__restrict__ ekin) {
  if (threadIdx.x == 0 && blockIdx.x == 0) th[0] += th[2] - *ekin;
}

// CSVR: per-block partial sums of the squares of ndof - 1 normal numbers
__global__ void k_csvr_chi2(int64_t m, unsigned long long seed, const int *__restrict__ step,
                            double *__restrict__ part) {
  __shared__ double red[8];
  double s = 0.0;
  for (int64_t t = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; t < m; t += (int64_t)gridDim.x * blockDim.x) {
    const double z = normal01(seed, (unsigned long long)t, *step, 3);
    s += z * z;
  }
#pragma unroll
  for (int o = 16; o > 0; o >>= 1) s += __shfl_xor_sync(0xffffffffu, s, o);
  if ((threadIdx.x & 31) == 0) red[threadIdx.x >> 5] = s;
  __syncthreads();
  if (threadIdx.x == 0) {
    double q = 0.0;
    for (int w = 0; w < (int)(blockDim.x >> 5); w++) q += red[w];
    part[blockIdx.x] = q;
  }
}

// CSVR rescaling factor alpha (nvt.py:255-265; Bussi and Parrinello, Comput.
// Phys. Commun. 179, 26 (2008)).
__global__ void k_csvr(double *__restrict__ th, double *__restrict__ ekin, double kT, double c, double ndof,
                       unsigned long long seed, const int *__restrict__ step) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  const double R = normal01(seed, 0xFFFFFFFFFFFFull, *step, 2);
  const double S = th[3];
  const double ek = *ekin;
  const double kin = 0.5 * ndof * kT;
  const double fact = (1.0 - c) * kin / ndof / ek;
  const double a2 = c + (S + R * R) * fact + 2.0 * R * sqrt(c * fact);
  const double alpha = (R + sqrt(c / fact) >= 0.0 ? 1.0 : -1.0) * sqrt(a2);
  th[1] = alpha;
  th[0] += (1.0 - alpha * alpha) * ek;
  *ekin = alpha * alpha * ek;
}

// One application of the Nose-Hoover chain propagator (nvt.py:378-417):
// chain velocities a quarter step (reverse order), chain positions half a
// step, the atomic velocity factor, chain velocities again (forward order).
// post = 1 also stores the chain's conserved-energy correction.
__global__ void k_nhc(double *__restrict__ th, double *__restrict__ ekin, int len, double dt, double kT, double ndof,
                      int post) {
  if (threadIdx.x != 0 || blockIdx.x != 0) return;
  double *xi = th + 8, *vxi = th + 16;
  const double *Q = th + 24;
  double ek = *ekin;
  for (int pass = 0; pass < 2; pass++) {
    for (int q = 0; q < len; q++) {
      const int k = pass == 0 ? len - 1 - q : q;
      double g = (k == 0) ? 2.0 * ek - ndof * kT : Q[k - 1] * vxi[k - 1] * vxi[k - 1] - kT;
      g /= Q[k];
      if (k == len - 1) {
        vxi[k] += g * dt / 4;
      } else {
        const double e = exp(-vxi[k + 1] * dt / 8);
        vxi[k] *= e;
        vxi[k] += g * dt / 4;
        vxi[k] *= e;
      }
    }
    if (pass == 0) {
      for (int k = 0; k < len; k++) xi[k] += vxi[k] * dt / 2;
      const double f = exp(-vxi[0] * dt / 2);
      th[1] = f;
      ek *= f * f;
    }
  }
  *ekin = ek;
  if (post) {
    double e = 0.0, x = ndof * xi[0];
    for (int k = 0; k < len; k++) e += vxi[k] * vxi[k] * Q[k];
    for (int k = 1; k < len; k++) x += xi[k];
    th[0] = 0.5 * e + kT * x;
  }
}

}  // namespace

// Thermostat stage of the device step: stage 0 before the first half kick
// (the reference's pre hook), 1 after the second (its post hook).
static int md_thermostat(yg_ctx *c, int stage) {
  if (!c->md_thermo) return YG_OK;
  const int64_t n3 = c->natom * 3;
  const int nb = yg_blocks(n3, 256);
  const double dt = c->md_dt, nd = (double)c->md_ndof;
  int rc;
  switch (c->md_thermo) {
    case 1:  // Berendsen: pre only
      if (stage != 0) return YG_OK;
      k_berendsen<<<1, 32, 0, c->stream>>>(c->d_md_thermo, c->d_md_ekin, c->md_kT, dt / c->md_timecon, nd);
      YG_LAUNCH_CHECK(c, "k_berendsen");
      break;
    case 2: {  // Langevin: pre and post
      k_save_ekin<<<1, 32, 0, c->stream>>>(c->d_md_thermo, c->d_md_ekin);
      YG_LAUNCH_CHECK(c, "k_save_ekin");
      k_langevin<<<nb, 256, 0, c->stream>>>(c->d_vel, c->d_invm, c->natom, exp(-dt / c->md_timecon / 2), c->md_kT,
                                            c->md_seed, c->d_md_step, stage, c->d_md_ekpart);
      YG_LAUNCH_CHECK(c, "k_langevin");
      if ((rc = yg_launch_reduce_ev(c, c->d_md_ekpart, nb, 1, c->d_md_ekin))) return rc;
      k_ekin_delta<<<1, 32, 0, c->stream>>>(c->d_md_thermo, c->d_md_ekin);
      YG_LAUNCH_CHECK(c, "k_ekin_delta");
      return YG_OK;
    }
    case 3: {  // CSVR: pre only
      if (stage != 0) return YG_OK;
      const int64_t m = c->md_ndof - 1;
      const int nbc = (int)std::max<int64_t>(1, std::min<int64_t>(yg_blocks(m, 256), nb));
      k_csvr_chi2<<<nbc, 256, 0, c->stream>>>(m, c->md_seed, c->d_md_step, c->d_md_ekpart);
      YG_LAUNCH_CHECK(c, "k_csvr_chi2");
      if ((rc = yg_launch_reduce_ev(c, c->d_md_ekpart, nbc, 1, c->d_md_thermo + 3))) return rc;
      k_csvr<<<1, 32, 0, c->stream>>>(c->d_md_thermo, c->d_md_ekin, c->md_kT, exp(-dt / c->md_timecon), nd,
                                      c->md_seed, c->d_md_step);
      YG_LAUNCH_CHECK(c, "k_csvr");
      break;
    }
    default:  // Nose-Hoover chain: pre and post
      k_nhc<<<1, 32, 0, c->stream>>>(c->d_md_thermo, c->d_md_ekin, c->md_nhc_len, dt, c->md_kT, nd, stage);
      YG_LAUNCH_CHECK(c, "k_nhc");
      break;
  }
  k_scale_vel<<<nb, 256, 0, c->stream>>>(c->d_vel, n3, c->d_md_thermo);
  YG_LAUNCH_CHECK(c, "k_scale_vel");
  return YG_OK;
}

// Force evaluation for the current device positions on the kept list,
// summed on the device into d_total; no host synchronization.  prep = 0
// when the cell-local coordinates are already current.
static int md_force_async(yg_ctx *c, int prep, int reci_forked) {
  int rc;
  if (prep && (rc = yg_launch_prep_positions(c))) return rc;
  if (!reci_forked && (c->md_mask & (1 << YG_PART_EWALD_RECI)) && (rc = yg_launch_ewald_reci(c, 1))) return rc;
  int pmask = 0;
  for (int p = 0; p < YG_MAX_POT; p++)
    if (c->pot[p].active && (c->md_mask & (1 << p))) pmask |= 1 << p;
  if (pmask && (rc = yg_launch_pair(c, pmask, 1))) return rc;
  if ((c->md_mask & (1 << YG_PART_EWALD_CORR)) && (rc = yg_launch_ewald_corr(c, 1))) return rc;
  if ((c->md_mask & (1 << YG_PART_VALENCE)) && (rc = yg_launch_valence(c, 1))) return rc;
  if ((rc = yg_ewald_join(c))) return rc;
  k_total_dev<<<yg_blocks(c->natom * 3, 256), 256, 0, c->stream>>>(c->d_part_ev, c->d_part_gpos, c->natom,
                                                                  c->md_mask, c->d_total);
  YG_LAUNCH_CHECK(c, "k_total_dev");
  return YG_OK;
}

// second kick, kinetic energy, post-step thermostat, energy log row
static int md_finish_step(yg_ctx *c, double dt, int thermo) {
  int rc;
  const int nb = yg_blocks(c->natom * 3, 256);
  k_kick<<<nb, 256, 0, c->stream>>>(c->d_vel, c->d_total + 16, c->d_invm, c->natom, dt, c->d_md_ekpart);
  YG_LAUNCH_CHECK(c, "k_kick");
  if ((rc = yg_launch_reduce_ev(c, c->d_md_ekpart, nb, 1, c->d_md_ekin))) return rc;
  if (thermo && (rc = md_thermostat(c, 1))) return rc;
  k_md_log<<<1, 32, 0, c->stream>>>(c->d_total, c->d_md_ekin, c->d_md_extra, c->d_md_log, c->d_md_step,
                                    c->md_max_steps + 1);
  YG_LAUNCH_CHECK(c, "k_md_log");
  return YG_OK;
}

// One whole step, enqueued without host synchronization.
static int md_step_device(yg_ctx *c, double factor, double skin) {
  int rc;
  const int nb = yg_blocks(c->natom * 3, 256);
  if ((rc = md_thermostat(c, 0))) return rc;
  k_kick_drift<<<nb, 256, 0, c->stream>>>(c->d_pos, c->d_vel, c->d_total + 16, c->d_invm, c->natom, c->md_dt);
  YG_LAUNCH_CHECK(c, "k_kick_drift");
  if ((rc = yg_launch_max_disp2_async(c, (unsigned long long *)(c->d_md_ctrl + 6)))) return rc;
  k_skin_gate<<<1, 32, 0, c->stream>>>(c->d_md_ctrl, factor, skin);
  YG_LAUNCH_CHECK(c, "k_skin_gate");
  // the reciprocal sum needs only the new positions: it runs on the
  // auxiliary stream while the list is rebuilt (when due) and the pair
  // terms are evaluated
  const int reci = (c->md_mask & (1 << YG_PART_EWALD_RECI)) != 0;
  if (reci && (rc = yg_launch_ewald_reci(c, 1))) return rc;
  // the build sequence refreshes the cell-local coordinates in any case
  if ((rc = yg_launch_nlist_build_gated(c, c->d_md_ctrl, (unsigned long long *)(c->d_md_ctrl + 4)))) return rc;
  // the pair terms read the skin shell of the rows only on steps without a rebuild
  c->pair_fresh_dev = c->d_md_ctrl;
  rc = md_force_async(c, 0, reci);
  c->pair_fresh_dev = nullptr;
  if (rc) return rc;
  return md_finish_step(c, c->md_dt, 1);
}

static void md_drop_graph(yg_ctx *c) {
  if (c->md_graph_exec) cudaGraphExecDestroy(c->md_graph_exec);
  c->md_graph_exec = nullptr;
  c->md_graph_valid = 0;
}

// Records one step into the context's graph (on a private stream: the legacy
// default stream cannot be captured; the graph is replayed on the context's
// own stream).
static int md_capture(yg_ctx *c, double factor, double skin) {
  md_drop_graph(c);
  if (!c->md_cap_stream) YG_CUDA(cudaStreamCreateWithFlags(&c->md_cap_stream, cudaStreamNonBlocking));
  cudaStream_t own = c->stream;
  cudaGraph_t g;
  YG_CUDA(cudaStreamBeginCapture(c->md_cap_stream, cudaStreamCaptureModeRelaxed));
  c->stream = c->md_cap_stream;
  const int64_t nalloc = c->alloc_calls;
  int crc = md_step_device(c, factor, skin);
  c->stream = own;
  cudaError_t ce = cudaStreamEndCapture(c->md_cap_stream, &g);
  if (crc) return crc;
  if (ce != cudaSuccess) return yg_cuda_fail(ce, "cudaStreamEndCapture");
  if (c->alloc_calls != nalloc) {
    cudaGraphDestroy(g);
    yg_set_error("a buffer was allocated while capturing the step");
    return YG_ERR_STATE;
  }
  ce = cudaGraphInstantiate(&c->md_graph_exec, g, 0);
  cudaGraphDestroy(g);
  if (ce != cudaSuccess) return yg_cuda_fail(ce, "cudaGraphInstantiate");
  c->md_graph_valid = 1;
  c->md_graph_skin = skin;
  return YG_OK;
}

extern "C" {

// Per-atom neighbour-slot capacity of the next builds (rounded up to 32,
// at least 32).  Builds that need more slots regrow as usual: the host build
// reruns, the device-resident MD rolls its batch back and reruns it.
int yg_nlist_set_capacity(yg_ctx *c, int64_t slots) {
  if (!c || slots < 1) return YG_ERR_ARG;
  int rc;
  if ((rc = yg_ewald_join(c))) return rc;
  int64_t cap = (std::max<int64_t>(slots, 32) + 31) / 32 * 32;
  c->nbr_cap = cap;
  if (c->nbr_cap * c->natom > c->nbr_alloc) {
    yg_free(c, (void **)&c->d_nbr);
    if ((rc = yg_alloc(c, (void **)&c->d_nbr, (size_t)(c->nbr_cap * c->natom) * sizeof(uint2)))) return rc;
    c->nbr_alloc = c->nbr_cap * c->natom;
  }
  md_drop_graph(c);  // the capacity is baked into a captured step
  // the rows in the slots were laid out with the old capacity: no kernel may
  // read them again; the host path rebuilds before its next use and the
  // device-resident MD rebuilds at its next step
  c->rows_valid = 0;
  if (c->md_ready) {
    k_set_int<<<1, 32, 0, c->stream>>>(c->d_md_ctrl + 1, 1);
    YG_LAUNCH_CHECK(c, "k_set_int");
  }
  return YG_OK;
}

int yg_md_setup(yg_ctx *c, const double *masses, const double *vel, double dt, int part_mask, double extra_energy,
                int64_t max_steps) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (c && c->build_pending) {
    const int wrc = yg_launch_nlist_build_wait(c);
    if (wrc) return wrc;
  }
  if (!c || !masses || !vel || !(dt > 0.0) || max_steps < 1) return YG_ERR_ARG;
  if (!c->have_list) {
    yg_set_error("yg_md_setup: build the neighbour list first");
    return YG_ERR_STATE;
  }
  const int64_t N = c->natom;
  std::vector<double> invm(N);
  for (int64_t i = 0; i < N; i++) {
    if (!(masses[i] > 0.0)) return YG_ERR_ARG;
    invm[i] = 1.0 / masses[i];
  }
  int rc;
  const int nb = yg_blocks(N * 3, 256);
  md_drop_graph(c);
  void **bufs[] = {(void **)&c->d_vel,      (void **)&c->d_invm,     (void **)&c->d_md_ekpart,
                   (void **)&c->d_md_ekin,  (void **)&c->d_md_log,   (void **)&c->d_md_extra,
                   (void **)&c->d_md_step,  (void **)&c->d_md_ctrl,  (void **)&c->d_snap_pos,
                   (void **)&c->d_snap_vel, (void **)&c->d_snap_total, (void **)&c->d_snap_step,
                   (void **)&c->d_md_thermo, (void **)&c->d_snap_thermo};
  for (void **b : bufs) yg_free(c, b);
  c->md_thermo = 0;
  if ((rc = yg_alloc(c, (void **)&c->d_vel, N * 3 * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_invm, N * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_md_ekpart, (size_t)nb * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_md_ekin, sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_md_log, (size_t)(max_steps + 1) * 2 * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_md_extra, sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_md_step, sizeof(int)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_md_ctrl, 16 * sizeof(int)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_snap_pos, N * 3 * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_snap_vel, N * 3 * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_snap_total, (16 + N * 3) * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_snap_step, sizeof(int)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_md_thermo, 40 * sizeof(double)))) return rc;
  if ((rc = yg_alloc(c, (void **)&c->d_snap_thermo, 40 * sizeof(double)))) return rc;
  YG_CUDA(cudaMemsetAsync(c->d_md_thermo, 0, 40 * sizeof(double), c->stream));
  YG_CUDA(cudaMemcpyAsync(c->d_vel, vel, N * 3 * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  YG_CUDA(cudaMemcpyAsync(c->d_invm, invm.data(), N * sizeof(double), cudaMemcpyHostToDevice, c->stream));
  YG_CUDA(cudaMemcpyAsync(c->d_md_extra, &extra_energy, sizeof(double), cudaMemcpyHostToDevice, c->stream));
  YG_CUDA(cudaMemsetAsync(c->d_md_step, 0, sizeof(int), c->stream));
  YG_CUDA(cudaMemsetAsync(c->d_md_ctrl, 0, 16 * sizeof(int), c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  c->md_dt = dt;
  c->md_mask = part_mask;
  c->md_max_steps = max_steps;
  c->md_steps_done = 0;
  c->md_rebuilds = 0;
  c->md_ready = 1;
  // step 0: forces and energies at the initial positions (yaff's initialize);
  // a kick with dt = 0 only evaluates the kinetic energy
  if ((rc = md_force_async(c, 1, 0))) return rc;
  return md_finish_step(c, 0.0, 0);
}

// Runs nsteps velocity-Verlet steps in batches of at most YG_MD_BATCH: each
// batch snapshots the state, enqueues its steps (graph replay when
// use_graph is set; the graph is captured on first use after one eager step
// and again whenever the neighbour slots were reallocated), then reads the
// status words once.  skin <= 0 rebuilds every step.
int yg_md_run(yg_ctx *c, int64_t nsteps, int use_graph, double skin, int64_t *nrebuild) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c || nsteps < 0) return YG_ERR_ARG;
  if (!c->md_ready) {
    yg_set_error("yg_md_run: call yg_md_setup first");
    return YG_ERR_STATE;
  }
  if (c->build_pending) {
    const int wrc = yg_launch_nlist_build_wait(c);
    if (wrc) return wrc;
  }
  if (c->md_steps_done + nsteps > c->md_max_steps) {
    yg_set_error("yg_md_run: more steps than the energy log holds");
    return YG_ERR_CAPACITY;
  }
  int rc;
  const int64_t rmaxmax = std::max(c->rmax[0], std::max(c->rmax[1], c->rmax[2]));
  const double factor = 2.0 * (double)(rmaxmax + 1);
  const int64_t N = c->natom;
  const int64_t reb0 = c->md_rebuilds;
  int64_t left = nsteps;
  int replays = 0;
  if (c->md_graph_valid && c->md_graph_skin != skin) md_drop_graph(c);  // the skin is baked into the graph
  while (left > 0) {
    const int64_t nb = std::min<int64_t>(left, YG_MD_BATCH);
    // snapshot
    YG_CUDA(cudaMemcpyAsync(c->d_snap_pos, c->d_pos, N * 3 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    YG_CUDA(cudaMemcpyAsync(c->d_snap_vel, c->d_vel, N * 3 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
    YG_CUDA(cudaMemcpyAsync(c->d_snap_total, c->d_total, (16 + N * 3) * sizeof(double), cudaMemcpyDeviceToDevice,
                            c->stream));
    YG_CUDA(cudaMemcpyAsync(c->d_snap_step, c->d_md_step, sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
    YG_CUDA(cudaMemcpyAsync(c->d_snap_thermo, c->d_md_thermo, 40 * sizeof(double), cudaMemcpyDeviceToDevice,
                            c->stream));
    YG_CUDA(cudaMemsetAsync(c->d_status, 0, YG_ST_NWORDS * sizeof(int), c->stream));
    for (int64_t s = 0; s < nb; s++) {
      if (use_graph && c->md_graph_valid) {
        YG_CUDA(cudaGraphLaunch(c->md_graph_exec, c->stream));
        c->launches++;
        continue;
      }
      // eager step (sizes every scratch buffer), then capture for the rest
      if ((rc = md_step_device(c, factor, skin))) return rc;
      if (use_graph) {
        YG_CUDA(cudaStreamSynchronize(c->stream));
        if ((rc = md_capture(c, factor, skin))) return rc;
      }
    }
    // one readback per batch: status words and control words
    YG_CUDA(cudaMemcpyAsync(c->h_status, c->d_status, YG_ST_NWORDS * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    YG_CUDA(cudaMemcpyAsync(c->h_u64, c->d_md_ctrl, 16 * sizeof(int), cudaMemcpyDeviceToHost, c->stream));
    YG_CUDA(cudaStreamSynchronize(c->stream));
    const int *ctrl = (const int *)c->h_u64;
    if (c->h_status[YG_ST_BADCELL]) {
      yg_set_error("non-finite or huge position met while rebuilding the neighbour list");
      return YG_ERR_NAN;
    }
    if (c->h_status[YG_ST_OVERFLOW]) {
      if (++replays > 8) {
        yg_set_error("neighbour slots kept overflowing during device rebuilds");
        return YG_ERR_CAPACITY;
      }
      // roll back to the snapshot, grow the slots, rebuild at the first step
      YG_CUDA(cudaMemcpyAsync(c->d_pos, c->d_snap_pos, N * 3 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      YG_CUDA(cudaMemcpyAsync(c->d_vel, c->d_snap_vel, N * 3 * sizeof(double), cudaMemcpyDeviceToDevice, c->stream));
      YG_CUDA(cudaMemcpyAsync(c->d_total, c->d_snap_total, (16 + N * 3) * sizeof(double), cudaMemcpyDeviceToDevice,
                              c->stream));
      YG_CUDA(cudaMemcpyAsync(c->d_md_step, c->d_snap_step, sizeof(int), cudaMemcpyDeviceToDevice, c->stream));
      YG_CUDA(cudaMemcpyAsync(c->d_md_thermo, c->d_snap_thermo, 40 * sizeof(double), cudaMemcpyDeviceToDevice,
                              c->stream));
      int64_t cap = (int64_t)(c->h_status[YG_ST_MAXCOUNT] * 1.15) + 64;
      cap = (cap + 31) / 32 * 32;
      if (cap > c->nbr_cap) c->nbr_cap = cap;
      if (c->nbr_cap * N > c->nbr_alloc) {
        yg_free(c, (void **)&c->d_nbr);
        if ((rc = yg_alloc(c, (void **)&c->d_nbr, (size_t)(c->nbr_cap * N) * sizeof(uint2)))) return rc;
        c->nbr_alloc = c->nbr_cap * N;
      }
      md_drop_graph(c);
      k_set_int<<<1, 32, 0, c->stream>>>(c->d_md_ctrl + 1, 1);
      YG_LAUNCH_CHECK(c, "k_set_int");
      k_set_int<<<1, 32, 0, c->stream>>>(c->d_md_ctrl + 2, (int)c->md_rebuilds);
      YG_LAUNCH_CHECK(c, "k_set_int");
      continue;
    }
    if (ctrl[2] != (int)c->md_rebuilds) c->nneigh = (int64_t)(c->h_u64[2] / 2);
    c->md_rebuilds = ctrl[2];
    c->md_steps_done += nb;
    left -= nb;
  }
  c->list_recomputed = 1;
  if (nsteps > 0) c->rows_valid = 1;  // a forced rebuild ran at the first step
  for (int p = 0; p < YG_NPART; p++) c->part_valid[p] = 0;
  if (nrebuild) *nrebuild = c->md_rebuilds - reb0;
  return YG_OK;
}

// Copies positions, velocities (natom x 3, may be NULL) and the energy log
// ((steps done + 1) x (epot, ekin), may be NULL) to host memory.
int yg_md_get(yg_ctx *c, double *pos, double *vel, double *log, int64_t *nlog) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c || !c->md_ready) return YG_ERR_STATE;
  if (pos) YG_CUDA(cudaMemcpyAsync(pos, c->d_pos, c->natom * 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  if (vel) YG_CUDA(cudaMemcpyAsync(vel, c->d_vel, c->natom * 3 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  const int64_t n = c->md_steps_done + 1;
  if (log) YG_CUDA(cudaMemcpyAsync(log, c->d_md_log, n * 2 * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  if (nlog) *nlog = n;
  if (log && std::isnan(log[2 * (n - 1)])) {
    yg_set_error("not-a-number energy in the trajectory");
    return YG_ERR_NAN;
  }
  return YG_OK;
}

int yg_md_thermostat(yg_ctx *c, int kind, double kT, double timecon, int64_t ndof, int chain_length,
                     const double *chain_pos, const double *chain_vel, const double *chain_masses,
                     unsigned long long seed) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c || kind < 0 || kind > 4) return YG_ERR_ARG;
  if (!c->md_ready) {
    yg_set_error("yg_md_thermostat: call yg_md_setup first");
    return YG_ERR_STATE;
  }
  if (kind != 0 && (!(kT > 0.0) || !(timecon > 0.0) || ndof < 2)) return YG_ERR_ARG;
  if (kind == 4 && (chain_length < 1 || chain_length > 8 || !chain_pos || !chain_vel || !chain_masses)) {
    yg_set_error("a Nose-Hoover chain needs 1..8 beads with positions, velocities and masses");
    return YG_ERR_ARG;
  }
  double h[40] = {0.0};
  if (kind == 4)
    for (int k = 0; k < chain_length; k++) {
      if (!(chain_masses[k] > 0.0)) return YG_ERR_ARG;
      h[8 + k] = chain_pos[k];
      h[16 + k] = chain_vel[k];
      h[24 + k] = chain_masses[k];
    }
  YG_CUDA(cudaMemcpyAsync(c->d_md_thermo, h, sizeof(h), cudaMemcpyHostToDevice, c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  c->md_thermo = kind;
  c->md_kT = kT;
  c->md_timecon = timecon;
  c->md_ndof = ndof;
  c->md_nhc_len = kind == 4 ? chain_length : 0;
  c->md_seed = seed;
  md_drop_graph(c);  // the step changed
  return YG_OK;
}

int yg_md_thermo_get(yg_ctx *c, double *econs_correction, double *chain_pos, double *chain_vel) {
  if (c) {
    const int jrc = yg_ewald_join(c);
    if (jrc) return jrc;
  }
  if (!c || !c->md_ready) return YG_ERR_STATE;
  double h[40];
  YG_CUDA(cudaMemcpyAsync(h, c->d_md_thermo, sizeof(h), cudaMemcpyDeviceToHost, c->stream));
  YG_CUDA(cudaStreamSynchronize(c->stream));
  if (econs_correction) *econs_correction = h[0];
  for (int k = 0; k < c->md_nhc_len; k++) {
    if (chain_pos) chain_pos[k] = h[8 + k];
    if (chain_vel) chain_vel[k] = h[16 + k];
  }
  return YG_OK;
}

}  // extern "C"
