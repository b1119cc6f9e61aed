// yg_fleet.cu -- many small periodic systems stepped together on one GPU.
//
// A fleet holds up to max_systems independent LJ + EI + Ewald systems (the
// serving workload: velocity Verlet of 64 .. a few thousand atoms each) in
// fixed-capacity device arrays: atoms of a system occupy a contiguous range
// (aligned to 128 atoms), its reciprocal vectors a contiguous range of the k
// table (aligned to 32), and a device table of per-system records holds the
// cell, cutoffs, counters and state.  One MD step of every system in flight
// is eight launches, whatever the number of systems:
//   drift     (atom)   first half kick and drift; displacement since the
//                      last build; fractional coordinates (FP32 hi + lo);
//                      the atom's phase tables exp(2 pi i g s) per axis
//   gate      (system) the reference's skin rule per system
//                      (yaff/pes/nlist.py:207-218)
//   build     (tile)   neighbour rows of the systems whose gate fired:
//                      128-atom tiles of the system staged in shared memory,
//                      every periodic image within rcut + skin; relative
//                      vectors as exact FP32 hi + lo differences of the
//                      wrapped Cartesian positions plus the image shift (hi +
//                      lo), rounded once: a row entry keeps them
//   pair      (atom)   LJ + real-space EI over the row in FP32, the relative
//                      vector refreshed by the displacements since the build
//                      (the reference's skin path, nlist.c:183-232)
//   sfac      (k)      structure factors S(k) of each system's half sphere
//                      (a block of 128 k vectors sweeps the system's atoms
//                      in tiles of 32 whose phase tables it stages in shared
//                      memory: a phase is two complex products), and the
//                      FP32 coefficients 2 A(k) S(k) of the gradient
//   ewald     (atom)   reciprocal-space gradient from those coefficients and
//                      the atom's own phase tables
//   kick      (atom)   total gradient, second half kick, kinetic energy
//   finish    (system) fixed-order energy sums, the log row, the counters
// Every reduction over a system runs inside that system's own threads in a
// fixed order, so a system's trajectory does not depend on which other
// systems are in flight.  The step is captured once into a CUDA graph and
// replayed; systems join and leave between replays by editing the tables.
// Physics: the reference's LJ (pair_pot.c:277-301), point-charge EI with
// Ewald screening (pair_pot.c:724-735), Ewald reciprocal sum
// (ewald.c:32-150), self and neutralizing terms (ewald.c:289-292,
// ff.py:633-669) and velocity Verlet (verlet.py:339-367); pair terms,
// phases and structure factors in FP32 with compensated sums, positions,
// velocities and energies in FP64.  No FP64 arithmetic runs per pair or per
// atom and k vector: the FP64 pipe of this part is a small fraction of its
// FP32 rate.  The neighbour decision at rcut + skin is FP32 (deterministic,
// so a system's list is the same alone and in a mix; pairs beyond rcut are
// masked by the pair kernel and the skin rule keeps the list complete).
#include <cmath>
#include <cstring>
#include <vector>

#include "yg_internal.cuh"
#include "yg_pairterm.cuh"

#define FL_TILE 128    // atoms per build tile and per atom-range granule
#define FL_KGRAN 128   // k-vector range granule (a structure-factor block lies in one system)
#define FL_TAB 64      // phase-table slots per atom: (G0 + 1) + (G1 + 1) + (G2 + 1) at most
#define FL_RMAX 2      // periodic images searched per axis, at most
#define FL_SHIFTS ((2 * FL_RMAX + 3) * (2 * FL_RMAX + 3) * (2 * FL_RMAX + 3))

struct FleetSys {
  int a0, n, k0, nk;
  int state;      // 0 empty, 1 stepping, 2 done, 3 failed (neighbour overflow)
  int init;       // 1 until the forces of step 0 are computed
  int rebuild;    // the gate fired this step
  int overflow;   // a row ran out of slots at the last build
  int rmax[3];    // periodic images searched per axis
  int gmax[3];    // reciprocal-lattice extent per axis (phase-table slots G + 1 each)
  int step;       // steps completed
  int nsteps;     // steps requested
  unsigned maxd2; // bits of the largest squared displacement since the last build (FP32, >= 0)
  double rv[9];   // cell vectors (rows)
  double gv[9];   // reciprocal vectors (rows)
  double rcut, rcs, alpha, dt, skin, e_const, epot, ekin;
};

// Device arrays of a fleet (kernel argument).
struct FleetDev {
  int cap, max_steps;
  // atoms
  double *pos, *vel, *pos_build, *invm, *gtot;
  double *gpair, *gew, *epair, *ekin;
  float *q, *sig, *seps;
  float4 *disp, *fhi, *flo;  // displacement since the build; fractional coordinates (hi, lo)
  float4 *chi, *clo;         // Cartesian position wrapped into the cell (hi, lo)
  int *sysid, *ncount;
  int4 *nbr;                // (j, FP32 relative vector at the build)
  // k vectors
  int4 *kg;                 // (g0, g1, g2, system or -1)
  float4 *kv;               // (kx, ky, kz, 0)
  float2 *kcoef;            // 2 A(k) S(k) as FP32 (written by the S pass)
  int *kslot;               // phase-table slots |g0|, off1 + |g1|, off2 + g2 (8 bits each), then
                            // bit 24: g0 < 0, bit 25: g1 < 0 (conjugate)
  float2 *ptab;             // [slot][atom] exp(2 pi i g s_axis), slot = axis offset + |g|
  int64_t acap;             // atom capacity (the slot stride of ptab)
  double *kpref;            // A(k) = 4 pi / V exp(-k^2 / 4 alpha^2) / k^2
  double2 *S;
  // systems
  FleetSys *d_sys;
  double *log;              // [system][max_steps + 1][2]
};

struct yg_fleet {
  int64_t max_atoms = 0, max_k = 0;
  int max_systems = 0;
  cudaStream_t stream = nullptr;
  int own_stream = 0;
  FleetDev d;
  std::vector<FleetSys> h_sys;
  FleetSys *h_sys_pinned = nullptr;
  // host bookkeeping of the free ranges (granules)
  std::vector<int> atom_owner, k_owner;
  // captured step
  cudaGraphExec_t graph = nullptr;
  cudaStream_t cap_stream = nullptr;
  int64_t launches = 0;
};

namespace {

__device__ __forceinline__ void kahan_add(float &s, float &c, float x) {
  const float y = x - c;
  const float t = s + y;
  c = (t - s) - y;
  s = t;
}

// fractional part of g * s (s = s_hi + s_lo), exact to about 1e-7 turns:
// the product error of the FP32 multiply is recovered with an FMA
__device__ __forceinline__ float frac_gs(float g, float sh, float sl) {
  const float pp = g * sh;
  const float e = fmaf(g, sh, -pp);
  return (pp - rintf(pp)) + fmaf(g, sl, e);
}

__global__ void k_fl_drift(FleetDev F, int64_t natom_cap) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= natom_cap) return;
  const int s = F.sysid[i];
  if (s < 0) return;
  FleetSys &S = F.d_sys[s];
  if (S.state != 1) return;
  double r[3], v[3];
  for (int k = 0; k < 3; k++) {
    r[k] = F.pos[3 * i + k];
    v[k] = F.vel[3 * i + k];
  }
  if (!S.init) {
    const double h = 0.5 * S.dt, im = F.invm[i];
    for (int k = 0; k < 3; k++) {
      v[k] -= h * F.gtot[3 * i + k] * im;
      r[k] += S.dt * v[k];
      F.vel[3 * i + k] = v[k];
      F.pos[3 * i + k] = r[k];
    }
  }
  float d[3];
  for (int k = 0; k < 3; k++) d[k] = (float)(r[k] - F.pos_build[3 * i + k]);
  F.disp[i] = make_float4(d[0], d[1], d[2], 0.f);
  const float d2 = d[0] * d[0] + d[1] * d[1] + d[2] * d[2];
  atomicMax(&S.maxd2, __float_as_uint(d2));
  float sh[3], sl[3];
  for (int k = 0; k < 3; k++) {
    const double fs = S.gv[3 * k] * r[0] + S.gv[3 * k + 1] * r[1] + S.gv[3 * k + 2] * r[2];
    sh[k] = (float)fs;
    sl[k] = (float)(fs - (double)sh[k]);
  }
  F.fhi[i] = make_float4(sh[0], sh[1], sh[2], 0.f);
  F.flo[i] = make_float4(sl[0], sl[1], sl[2], 0.f);
  // phase tables: g s reduced exactly mod 1 (frac_gs), then one sincospi
  {
    int off = 0;
    for (int k = 0; k < 3; k++) {
      for (int g = 0; g <= S.gmax[k]; g++) {
        float sn, cs;
        sincospif(2.0f * frac_gs((float)g, sh[k], sl[k]), &sn, &cs);
        F.ptab[(int64_t)(off + g) * F.acap + i] = make_float2(cs, sn);
      }
      off += S.gmax[k] + 1;
    }
  }
  // the position wrapped into the cell, as FP32 hi + lo
  double fl[3], rw[3];
  for (int k = 0; k < 3; k++) fl[k] = floor(S.gv[3 * k] * r[0] + S.gv[3 * k + 1] * r[1] + S.gv[3 * k + 2] * r[2]);
  for (int x = 0; x < 3; x++) rw[x] = r[x] - (fl[0] * S.rv[x] + fl[1] * S.rv[3 + x] + fl[2] * S.rv[6 + x]);
  float ch[3], cl[3];
  for (int x = 0; x < 3; x++) {
    ch[x] = (float)rw[x];
    cl[x] = (float)(rw[x] - (double)ch[x]);
  }
  F.chi[i] = make_float4(ch[0], ch[1], ch[2], 0.f);
  F.clo[i] = make_float4(cl[0], cl[1], cl[2], 0.f);
}

__global__ void k_fl_gate(FleetDev F, int nsys) {
  const int s = blockIdx.x * blockDim.x + threadIdx.x;
  if (s >= nsys) return;
  FleetSys &S = F.d_sys[s];
  if (S.state != 1) return;
  const int rm = max(S.rmax[0], max(S.rmax[1], S.rmax[2]));
  const double disp = sqrt((double)__uint_as_float(S.maxd2));
  S.rebuild = (S.init || S.skin <= 0.0 || 2.0 * (rm + 1) * disp >= S.skin) ? 1 : 0;
  S.maxd2 = 0u;
}

// x + y = s + e exactly (Knuth's TwoSum; no operation may be reassociated)
__device__ __forceinline__ void two_sum(float x, float y, float &s, float &e) {
  s = x + y;
  const float bb = s - x;
  e = (x - (s - bb)) + (y - bb);
}

// One block per 128-atom tile; rows of the tile's atoms against every atom of
// the system and every image within rcut + skin.  The difference of two
// wrapped positions is exact as a + c (TwoSum of the hi parts, plus the lo
// parts); its FP32 fractional part picks the wrap w, and each image n adds
// the shift (n - w).R, tabulated per block as FP32 hi + lo from FP64.  A
// quick FP32 test of a + shift_hi selects the candidates whose vector is then
// summed with its error terms and rounded once.
__global__ void __launch_bounds__(FL_TILE) k_fl_build(FleetDev F, int64_t ntile) {
  __shared__ float4 sh[FL_TILE], sl[FL_TILE];
  __shared__ float4 th[FL_SHIFTS], tl[FL_SHIFTS];
  const int64_t t = blockIdx.x;
  if (t >= ntile) return;
  const int64_t i0 = t * FL_TILE;
  const int s = F.sysid[i0];
  if (s < 0) return;
  FleetSys &S = F.d_sys[s];
  if (S.state != 1 || !S.rebuild) return;
  const int r0 = S.rmax[0], r1 = S.rmax[1], r2 = S.rmax[2];
  const int W0 = 2 * r0 + 3, W1 = 2 * r1 + 3, W2 = 2 * r2 + 3;  // m = n - w in [-(r+1), r+1]
  for (int q = threadIdx.x; q < W0 * W1 * W2; q += FL_TILE) {
    const double m0 = q % W0 - (r0 + 1), m1 = (q / W0) % W1 - (r1 + 1), m2 = q / (W0 * W1) - (r2 + 1);
    float h[3], l[3];
    for (int x = 0; x < 3; x++) {
      const double v = m0 * S.rv[x] + m1 * S.rv[3 + x] + m2 * S.rv[6 + x];
      h[x] = (float)v;
      l[x] = (float)(v - (double)h[x]);
    }
    th[q] = make_float4(h[0], h[1], h[2], 0.f);
    tl[q] = make_float4(l[0], l[1], l[2], 0.f);
  }
  const int64_t a0 = S.a0, a1 = S.a0 + S.n;
  const int64_t i = i0 + threadIdx.x;
  const bool vi = i < a1;
  const float4 hi = vi ? F.chi[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float4 lo = vi ? F.clo[i] : make_float4(0.f, 0.f, 0.f, 0.f);
  const float rcs2 = (float)(S.rcs * S.rcs);
  const float rcs2q = (float)(S.rcs * S.rcs * (1.0 + 1e-4));
  const int cap = F.cap;
  float gf[9];
  for (int k = 0; k < 9; k++) gf[k] = (float)S.gv[k];
  int count = 0;
  int4 *row = F.nbr + i * cap;
  for (int64_t jt = a0; jt < a1; jt += FL_TILE) {
    const int64_t jl = jt + threadIdx.x;
    sh[threadIdx.x] = jl < a1 ? F.chi[jl] : make_float4(0.f, 0.f, 0.f, 0.f);
    sl[threadIdx.x] = jl < a1 ? F.clo[jl] : make_float4(0.f, 0.f, 0.f, 0.f);
    __syncthreads();
    const int nj = (int)(a1 - jt < FL_TILE ? a1 - jt : FL_TILE);
    if (vi) {
      for (int jj = 0; jj < nj; jj++) {
        const float4 hj = sh[jj], lj = sl[jj];
        float a[3], c[3];
        two_sum(hj.x, -hi.x, a[0], c[0]);
        two_sum(hj.y, -hi.y, a[1], c[1]);
        two_sum(hj.z, -hi.z, a[2], c[2]);
        c[0] += lj.x - lo.x;
        c[1] += lj.y - lo.y;
        c[2] += lj.z - lo.z;
        int w[3];
        for (int k = 0; k < 3; k++) w[k] = __float2int_rn(gf[3 * k] * a[0] + gf[3 * k + 1] * a[1] + gf[3 * k + 2] * a[2]);
        const int j = (int)(jt + jj);
        for (int n2 = -r2; n2 <= r2; n2++)
          for (int n1 = -r1; n1 <= r1; n1++)
            for (int n0 = -r0; n0 <= r0; n0++) {
              const int m0 = n0 - w[0], m1 = n1 - w[1], m2 = n2 - w[2];
              if (m0 < -(r0 + 1) || m0 > r0 + 1 || m1 < -(r1 + 1) || m1 > r1 + 1 || m2 < -(r2 + 1) || m2 > r2 + 1)
                continue;  // (an image beyond the searched range: never within rcut + skin)
              const int q = (m0 + r0 + 1) + W0 * ((m1 + r1 + 1) + W1 * (m2 + r2 + 1));
              const float4 Th = th[q];
              const float qx = a[0] + Th.x, qy = a[1] + Th.y, qz = a[2] + Th.z;
              if (!(qx * qx + qy * qy + qz * qz < rcs2q)) continue;
              const float4 Tl = tl[q];
              float ex, ey, ez, e0, e1, e2;
              two_sum(a[0], Th.x, ex, e0);
              two_sum(a[1], Th.y, ey, e1);
              two_sum(a[2], Th.z, ez, e2);
              ex += e0 + (c[0] + Tl.x);
              ey += e1 + (c[1] + Tl.y);
              ez += e2 + (c[2] + Tl.z);
              const float d2 = ex * ex + ey * ey + ez * ez;
              if (!(d2 < rcs2) || d2 == 0.f) continue;  // outside, or the atom itself
              if (count < cap)
                row[count] = make_int4(j, __float_as_int(ex), __float_as_int(ey), __float_as_int(ez));
              count++;
            }
      }
    }
    __syncthreads();
  }
  if (vi) {
    F.ncount[i] = min(count, cap);
    if (count > cap) atomicOr(&S.overflow, 1);
    for (int k = 0; k < 3; k++) F.pos_build[3 * i + k] = F.pos[3 * i + k];
    F.disp[i] = make_float4(0.f, 0.f, 0.f, 0.f);
  }
}

// LJ + real-space EI of every atom over its row, FP32 terms, compensated sums.
__global__ void k_fl_pair(FleetDev F, int64_t natom_cap) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= natom_cap) return;
  const int s = F.sysid[i];
  if (s < 0) return;
  const FleetSys &S = F.d_sys[s];
  if (S.state != 1) return;
  const float rc2 = (float)(S.rcut * S.rcut), alpha = (float)S.alpha;
  const float4 di = F.disp[i];
  const float qi = F.q[i], sgi = F.sig[i], sei = F.seps[i];
  float gx = 0.f, gy = 0.f, gz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f, e = 0.f, ce = 0.f;
  const int n = F.ncount[i];
  const int4 *row = F.nbr + i * F.cap;
  for (int k = 0; k < n; k++) {
    const int4 ent = row[k];
    const int j = ent.x;
    const float4 dj = F.disp[j];
    const float dx = __int_as_float(ent.y) + (dj.x - di.x);
    const float dy = __int_as_float(ent.z) + (dj.y - di.y);
    const float dz = __int_as_float(ent.w) + (dj.z - di.z);
    const float d2 = dx * dx + dy * dy + dz * dz;
    if (!(d2 < rc2)) continue;
    const float inv_d = rsqrtf(d2);
    const float d = d2 * inv_d, inv_d2 = inv_d * inv_d;
    float v = 0.f, g = 0.f;
    const float sig = 0.5f * (sgi + F.sig[j]), eps = sei * F.seps[j];
    if (eps != 0.f) {
      const float s2 = sig * sig * inv_d2;
      const float x = s2 * s2 * s2;
      g = 24.0f * eps * inv_d2 * x * (1.0f - 2.0f * x);
      v = 4.0f * eps * (x * (x - 1.0f));
    }
    const float qq = qi * F.q[j];
    if (qq != 0.f) {
      const float x = alpha * d;
      const float ve = qq * erfc_cheb(x) * inv_d;
      g += (-1.1283791670955126f * alpha * expf(-x * x) * qq - ve) * inv_d2;
      v += ve;
    }
    // gradient on i: -g * (r_j - r_i)
    kahan_add(gx, cx, -g * dx);
    kahan_add(gy, cy, -g * dy);
    kahan_add(gz, cz, -g * dz);
    kahan_add(e, ce, 0.5f * v);
  }
  F.gpair[3 * i] = (double)gx - (double)cx;
  F.gpair[3 * i + 1] = (double)gy - (double)cy;
  F.gpair[3 * i + 2] = (double)gz - (double)cz;
  F.epair[i] = (double)e - (double)ce;
}

// The phase exp(i k.r) of a k vector from an atom's tables (conjugates for
// negative g0, g1): two complex products.
__device__ __forceinline__ float2 fl_phase(float2 e0, float2 e1, float2 e2, int ks) {
  const float y0 = (ks >> 24) & 1 ? -e0.y : e0.y, y1 = (ks >> 25) & 1 ? -e1.y : e1.y;
  const float pr = e0.x * e1.x - y0 * y1, pi = e0.x * y1 + y0 * e1.x;
  return make_float2(pr * e2.x - pi * e2.y, pr * e2.y + pi * e2.x);
}

// S(k) of 128 reciprocal vectors of one system per block (k ranges are
// aligned to 128); the system's atoms are swept in tiles of 32 whose phase
// tables and charges are staged in shared memory.  Then the FP32
// coefficients 2 A(k) S(k) that the gradient pass reads.
__global__ void __launch_bounds__(128) k_fl_sfac(FleetDev F, int64_t nk_cap) {
  __shared__ float2 tab[FL_TAB][33];
  __shared__ float sq[32];
  const int64_t kb = (int64_t)blockIdx.x * 128;
  if (kb >= nk_cap) return;
  const int s = F.kg[kb].w;
  if (s < 0) return;
  const FleetSys &S = F.d_sys[s];
  if (S.state != 1) return;
  const int64_t kk = kb + threadIdx.x;
  const bool mine = F.kg[kk].w == s;  // the rest of the granule is padding
  const int ks = mine ? F.kslot[kk] : 0;
  const int s0 = ks & 255, s1 = (ks >> 8) & 255, s2 = (ks >> 16) & 255;
  const int ntab = S.gmax[0] + S.gmax[1] + S.gmax[2] + 3;
  const int64_t a1 = (int64_t)S.a0 + S.n;
  float cr = 0.f, ci = 0.f, kr = 0.f, ki = 0.f;
  for (int64_t at = S.a0; at < a1; at += 32) {
    const int na = (int)(a1 - at < 32 ? a1 - at : 32);
    for (int idx = threadIdx.x; idx < ntab * 32; idx += 128) {
      const int sl = idx >> 5, a = idx & 31;
      tab[sl][a] = a < na ? F.ptab[(int64_t)sl * F.acap + at + a] : make_float2(0.f, 0.f);
    }
    if (threadIdx.x < 32) sq[threadIdx.x] = (int)threadIdx.x < na ? F.q[at + threadIdx.x] : 0.f;
    __syncthreads();
    for (int a = 0; a < na; a++) {
      const float2 p = fl_phase(tab[s0][a], tab[s1][a], tab[s2][a], ks);
      const float qa = sq[a];
      kahan_add(cr, kr, qa * p.x);
      kahan_add(ci, ki, qa * p.y);
    }
    __syncthreads();
  }
  if (!mine) return;
  const double sr = (double)cr - (double)kr, si = (double)ci - (double)ki, a2 = 2.0 * F.kpref[kk];
  F.S[kk] = make_double2(sr, si);
  F.kcoef[kk] = make_float2((float)(a2 * sr), (float)(a2 * si));
}

// Reciprocal-space gradient of every atom of a 128-atom tile (one system)
// from its own phase tables and the system's coefficients, staged 128 k
// vectors at a time.
__global__ void __launch_bounds__(128) k_fl_ewald(FleetDev F, int64_t natom_cap) {
  __shared__ int sks[128];
  __shared__ float4 skv[128];
  __shared__ float2 scf[128];
  const int64_t i0 = (int64_t)blockIdx.x * 128;
  if (i0 >= natom_cap) return;
  const int s = F.sysid[i0];
  if (s < 0) return;
  const FleetSys &S = F.d_sys[s];
  if (S.state != 1) return;
  const int64_t i = i0 + threadIdx.x;
  const bool vi = i < (int64_t)S.a0 + S.n;
  const float qi = vi ? F.q[i] : 0.f;
  const float2 *pt = F.ptab + i;
  float gx = 0.f, gy = 0.f, gz = 0.f, cx = 0.f, cy = 0.f, cz = 0.f;
  int key01 = -1;
  float2 p01 = make_float2(0.f, 0.f);
  const int64_t k1 = (int64_t)S.k0 + S.nk;
  for (int64_t kc = S.k0; kc < k1; kc += 128) {
    const int nkc = (int)(k1 - kc < 128 ? k1 - kc : 128);
    if ((int)threadIdx.x < nkc) {
      sks[threadIdx.x] = F.kslot[kc + threadIdx.x];
      skv[threadIdx.x] = F.kv[kc + threadIdx.x];
      scf[threadIdx.x] = F.kcoef[kc + threadIdx.x];
    }
    __syncthreads();
    if (vi && qi != 0.f) {
      for (int q = 0; q < nkc; q++) {
        const int ks = sks[q];
        // consecutive k vectors of a (g0, g1) column share e0 e1 (the
        // test is uniform over the block)
        if ((ks & 0x0300ffff) != key01) {
          key01 = ks & 0x0300ffff;
          const float2 e0 = pt[(int64_t)(ks & 255) * F.acap], e1 = pt[(int64_t)((ks >> 8) & 255) * F.acap];
          const float y0 = (ks >> 24) & 1 ? -e0.y : e0.y, y1 = (ks >> 25) & 1 ? -e1.y : e1.y;
          p01 = make_float2(e0.x * e1.x - y0 * y1, e0.x * y1 + y0 * e1.x);
        }
        const float2 e2 = pt[(int64_t)((ks >> 16) & 255) * F.acap];
        const float2 p = make_float2(p01.x * e2.x - p01.y * e2.y, p01.x * e2.y + p01.y * e2.x);
        const float2 c = scf[q];
        const float4 k = skv[q];
        const float x = qi * (c.y * p.x - c.x * p.y);
        kahan_add(gx, cx, k.x * x);
        kahan_add(gy, cy, k.y * x);
        kahan_add(gz, cz, k.z * x);
      }
    }
    __syncthreads();
  }
  if (!vi) return;
  F.gew[3 * i] = (double)gx - (double)cx;
  F.gew[3 * i + 1] = (double)gy - (double)cy;
  F.gew[3 * i + 2] = (double)gz - (double)cz;
}

__global__ void k_fl_kick(FleetDev F, int64_t natom_cap) {
  const int64_t i = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (i >= natom_cap) return;
  const int s = F.sysid[i];
  if (s < 0) return;
  const FleetSys &S = F.d_sys[s];
  if (S.state != 1) return;
  const double im = F.invm[i], h = 0.5 * S.dt;
  double ek = 0.0;
  for (int k = 0; k < 3; k++) {
    const double g = F.gpair[3 * i + k] + F.gew[3 * i + k];
    F.gtot[3 * i + k] = g;
    double v = F.vel[3 * i + k];
    if (!S.init) {
      v -= h * g * im;
      F.vel[3 * i + k] = v;
    }
    ek += v * v;
  }
  F.ekin[i] = 0.5 * ek / im;
}

// One block per system: energies of the step in a fixed order, the log row,
// the counters.
__global__ void k_fl_finish(FleetDev F, int nsys) {
  __shared__ double red[3][256];
  const int s = blockIdx.x;
  if (s >= nsys) return;
  FleetSys &S = F.d_sys[s];
  if (S.state != 1) return;
  double ep = 0.0, ek = 0.0, er = 0.0;
  for (int64_t a = S.a0 + threadIdx.x; a < S.a0 + S.n; a += blockDim.x) {
    ep += F.epair[a];
    ek += F.ekin[a];
  }
  for (int64_t kk = S.k0 + threadIdx.x; kk < S.k0 + S.nk; kk += blockDim.x) {
    const double2 Sk = F.S[kk];
    er += F.kpref[kk] * (Sk.x * Sk.x + Sk.y * Sk.y);
  }
  red[0][threadIdx.x] = ep;
  red[1][threadIdx.x] = ek;
  red[2][threadIdx.x] = er;
  __syncthreads();
  for (int w = blockDim.x / 2; w > 0; w >>= 1) {
    if (threadIdx.x < w)
      for (int q = 0; q < 3; q++) red[q][threadIdx.x] += red[q][threadIdx.x + w];
    __syncthreads();
  }
  if (threadIdx.x == 0) {
    const double epot = red[0][0] + red[2][0] + S.e_const;
    S.epot = epot;
    S.ekin = red[1][0];
    if (S.init)
      S.init = 0;
    else
      S.step += 1;
    double *lg = F.log + ((int64_t)s * (F.max_steps + 1) + S.step) * 2;
    lg[0] = epot;
    lg[1] = red[1][0];
    if (S.overflow)
      S.state = 3;
    else if (S.step >= S.nsteps)
      S.state = 2;
  }
}

void fl_free(yg_fleet *f) {
  void *bufs[] = {f->d.pos, f->d.vel, f->d.pos_build, f->d.invm, f->d.gtot, f->d.gpair, f->d.gew, f->d.epair, f->d.ekin, f->d.q,
                  f->d.sig, f->d.seps, f->d.disp, f->d.fhi, f->d.flo, f->d.chi, f->d.clo, f->d.sysid, f->d.ncount, f->d.nbr, f->d.kg, f->d.kcoef,
                  f->d.kslot, f->d.ptab, f->d.kv, f->d.kpref, f->d.S, f->d.d_sys, f->d.log};
  for (void *b : bufs)
    if (b) cudaFree(b);
  if (f->h_sys_pinned) cudaFreeHost(f->h_sys_pinned);
  if (f->graph) cudaGraphExecDestroy(f->graph);
  if (f->cap_stream) cudaStreamDestroy(f->cap_stream);
  if (f->own_stream && f->stream) cudaStreamDestroy(f->stream);
}

int fl_launch_step(yg_fleet *f, cudaStream_t st) {
  const int64_t A = f->max_atoms, K = f->max_k;
  const int nb = (int)((A + 255) / 256);
  k_fl_drift<<<nb, 256, 0, st>>>(f->d, A);
  k_fl_gate<<<(f->max_systems + 127) / 128, 128, 0, st>>>(f->d, f->max_systems);
  k_fl_build<<<(int)(A / FL_TILE), FL_TILE, 0, st>>>(f->d, A / FL_TILE);
  k_fl_pair<<<nb, 256, 0, st>>>(f->d, A);
  k_fl_sfac<<<(int)(K / 128), 128, 0, st>>>(f->d, K);
  k_fl_ewald<<<(int)(A / 128), 128, 0, st>>>(f->d, A);
  k_fl_kick<<<nb, 256, 0, st>>>(f->d, A);
  k_fl_finish<<<f->max_systems, 256, 0, st>>>(f->d, f->max_systems);
  cudaError_t e = cudaGetLastError();
  if (e != cudaSuccess) return yg_cuda_fail(e, "fleet step");
  return YG_OK;
}

// first free run of `need` granules in an owner table (-1 = free), or -1
int fl_find(const std::vector<int> &own, int need) {
  int run = 0;
  for (int g = 0; g < (int)own.size(); g++) {
    run = own[g] < 0 ? run + 1 : 0;
    if (run == need) return g - need + 1;
  }
  return -1;
}

}  // namespace

extern "C" {

int yg_fleet_create(int64_t max_atoms, int max_systems, int64_t max_k, int max_neighbors, int max_steps,
                    void *stream, yg_fleet **out) {
  if (!out || max_atoms < FL_TILE || max_systems < 1 || max_k < FL_KGRAN || max_neighbors < 32 || max_steps < 1)
    return YG_ERR_ARG;
  *out = nullptr;
  yg_fleet *f = new yg_fleet();
  f->max_atoms = (max_atoms + FL_TILE - 1) / FL_TILE * FL_TILE;
  f->max_k = (max_k + FL_KGRAN - 1) / FL_KGRAN * FL_KGRAN;
  f->max_systems = max_systems;
  f->d.cap = (max_neighbors + 31) / 32 * 32;
  f->d.acap = f->max_atoms;
  f->d.max_steps = max_steps;
  if (stream) {
    f->stream = (cudaStream_t)stream;
  } else {
    if (cudaStreamCreateWithFlags(&f->stream, cudaStreamNonBlocking) != cudaSuccess) {
      delete f;
      yg_set_error("yg_fleet_create: cannot create a stream");
      return YG_ERR_CUDA;
    }
    f->own_stream = 1;
  }
  const int64_t A = f->max_atoms, K = f->max_k;
  const size_t Au = (size_t)f->max_atoms, Ku = (size_t)f->max_k;
  struct Buf { void **p; size_t bytes; } bufs[] = {
      {(void **)&f->d.pos, Au * 24}, {(void **)&f->d.vel, Au * 24}, {(void **)&f->d.pos_build, Au * 24},
      {(void **)&f->d.invm, Au * 8}, {(void **)&f->d.gtot, Au * 24}, {(void **)&f->d.gpair, Au * 24},
      {(void **)&f->d.gew, Au * 24}, {(void **)&f->d.epair, Au * 8}, {(void **)&f->d.ekin, Au * 8},
      {(void **)&f->d.q, Au * 4}, {(void **)&f->d.sig, Au * 4}, {(void **)&f->d.seps, Au * 4},
      {(void **)&f->d.disp, Au * 16}, {(void **)&f->d.chi, Au * 16}, {(void **)&f->d.clo, Au * 16}, {(void **)&f->d.fhi, Au * 16},
      {(void **)&f->d.flo, Au * 16}, {(void **)&f->d.sysid, Au * 4}, {(void **)&f->d.ncount, Au * 4},
      {(void **)&f->d.nbr, (size_t)Au * f->d.cap * 16}, {(void **)&f->d.kg, Ku * 16}, {(void **)&f->d.kcoef, Ku * 8},
      {(void **)&f->d.kslot, Ku * 4}, {(void **)&f->d.ptab, Au * FL_TAB * 8}, {(void **)&f->d.kv, Ku * 16},
      {(void **)&f->d.kpref, Ku * 8}, {(void **)&f->d.S, Ku * 16}, {(void **)&f->d.d_sys, (size_t)max_systems * sizeof(FleetSys)},
      {(void **)&f->d.log, (size_t)max_systems * (max_steps + 1) * 16}};
  for (auto &b : bufs) {
    cudaError_t e = cudaMalloc(b.p, b.bytes);
    if (e != cudaSuccess) {
      fl_free(f);
      delete f;
      yg_set_error("yg_fleet_create: device memory for the fleet could not be allocated");
      return YG_ERR_CUDA;
    }
  }
  cudaMemsetAsync(f->d.sysid, 0xff, A * 4, f->stream);
  cudaMemsetAsync(f->d.kg, 0xff, K * 16, f->stream);
  cudaMemsetAsync(f->d.d_sys, 0, (size_t)max_systems * sizeof(FleetSys), f->stream);
  cudaMemsetAsync(f->d.ncount, 0, A * 4, f->stream);
  if (cudaMallocHost(&f->h_sys_pinned, (size_t)max_systems * sizeof(FleetSys)) != cudaSuccess ||
      cudaStreamSynchronize(f->stream) != cudaSuccess) {
    fl_free(f);
    delete f;
    yg_set_error("yg_fleet_create: set-up failed");
    return YG_ERR_CUDA;
  }
  f->h_sys.assign(max_systems, FleetSys());
  std::memset(f->h_sys.data(), 0, sizeof(FleetSys) * max_systems);
  f->atom_owner.assign(A / FL_TILE, -1);
  f->k_owner.assign(K / FL_KGRAN, -1);
  *out = f;
  return YG_OK;
}

int yg_fleet_destroy(yg_fleet *f) {
  if (!f) return YG_ERR_ARG;
  cudaStreamSynchronize(f->stream);
  fl_free(f);
  delete f;
  return YG_OK;
}

int yg_fleet_add(yg_fleet *f, int64_t natom, const double *pos, const double *vel, const double *masses,
                 const double *charges, const double *sigma, const double *epsilon, const double *rvecs, double rcut,
                 double skin, double alpha, double gcut, double dt, int64_t nsteps, int *slot) {
  if (!f || natom < 1 || !pos || !vel || !masses || !charges || !sigma || !epsilon || !rvecs || !slot ||
      !(rcut > 0.0) || skin < 0.0 || !(alpha > 0.0) || !(gcut > 0.0) || !(dt > 0.0) || nsteps < 1)
    return YG_ERR_ARG;
  if (nsteps > f->d.max_steps) {
    yg_set_error("yg_fleet_add: more steps than the fleet's log holds");
    return YG_ERR_CAPACITY;
  }
  // free slot, atom range and k range
  int s = -1;
  for (int k = 0; k < f->max_systems; k++)
    if (f->h_sys[k].state == 0) {
      s = k;
      break;
    }
  if (s < 0) {
    yg_set_error("yg_fleet_add: every system slot is in use");
    return YG_ERR_CAPACITY;
  }
  // cell (the reference's SVD completion is not needed: three vectors)
  double R[9], G[9];
  std::memcpy(R, rvecs, sizeof(R));
  const double det = R[0] * (R[4] * R[8] - R[5] * R[7]) - R[1] * (R[3] * R[8] - R[5] * R[6]) +
                     R[2] * (R[3] * R[7] - R[4] * R[6]);
  if (!(std::fabs(det) > 0.0)) return YG_ERR_ARG;
  // G = inv(R)^T: rows g_k with g_k . r_l = delta_kl
  G[0] = (R[4] * R[8] - R[5] * R[7]) / det;
  G[1] = (R[5] * R[6] - R[3] * R[8]) / det;
  G[2] = (R[3] * R[7] - R[4] * R[6]) / det;
  G[3] = (R[2] * R[7] - R[1] * R[8]) / det;
  G[4] = (R[0] * R[8] - R[2] * R[6]) / det;
  G[5] = (R[1] * R[6] - R[0] * R[7]) / det;
  G[6] = (R[1] * R[5] - R[2] * R[4]) / det;
  G[7] = (R[2] * R[3] - R[0] * R[5]) / det;
  G[8] = (R[0] * R[4] - R[1] * R[3]) / det;
  const double volume = std::fabs(det);
  int rmax[3], gmax[3];
  for (int k = 0; k < 3; k++) {
    const double rsp = 1.0 / std::sqrt(G[3 * k] * G[3 * k] + G[3 * k + 1] * G[3 * k + 1] + G[3 * k + 2] * G[3 * k + 2]);
    const double gsp = 1.0 / std::sqrt(R[3 * k] * R[3 * k] + R[3 * k + 1] * R[3 * k + 1] + R[3 * k + 2] * R[3 * k + 2]);
    rmax[k] = (int)std::ceil((rcut + skin) / rsp - 0.5);
    gmax[k] = (int)std::ceil(gcut / gsp - 0.5);
    if (k == 2 && gmax[0] + gmax[1] + gmax[2] + 3 > FL_TAB) {
      yg_set_error("yg_fleet_add: too many reciprocal vectors per axis for the phase tables (raise the Ewald "
                   "alpha or lower gcut)");
      return YG_ERR_ARG;
    }
    if (rmax[k] > FL_RMAX) {
      yg_set_error("yg_fleet_add: the cell is too small for rcut + skin (more than two periodic images per axis)");
      return YG_ERR_ARG;
    }
  }
  // the half sphere of k vectors (yaff/pes/ewald.c:54-64) and A(k)
  const double tp = 6.2831853071795864769, fp = 12.566370614359172954;
  const double fac1 = fp / volume, fac2 = 0.25 / alpha / alpha;
  double gc2 = gcut * tp;
  gc2 *= gc2;
  std::vector<int4> kg;
  std::vector<float4> kv;
  std::vector<int> ksl;
  std::vector<double> kp;
  for (int g0 = -gmax[0]; g0 <= gmax[0]; g0++)
    for (int g1 = -gmax[1]; g1 <= gmax[1]; g1++)
      for (int g2 = 0; g2 <= gmax[2]; g2++) {
        if (g2 == 0 && (g1 < 0 || (g1 == 0 && g0 <= 0))) continue;
        double k[3];
        for (int x = 0; x < 3; x++) k[x] = tp * (g0 * G[x] + g1 * G[3 + x] + g2 * G[6 + x]);
        const double ksq = k[0] * k[0] + k[1] * k[1] + k[2] * k[2];
        if (ksq > gc2) continue;
        kg.push_back(make_int4(g0, g1, g2, s));
        kv.push_back(make_float4((float)k[0], (float)k[1], (float)k[2], 0.f));
        ksl.push_back(std::abs(g0) | ((gmax[0] + 1 + std::abs(g1)) << 8) | ((gmax[0] + gmax[1] + 2 + g2) << 16) |
                      ((g0 < 0) << 24) | ((g1 < 0) << 25));
        kp.push_back(fac1 * std::exp(-ksq * fac2) / ksq);
      }
  const int ag = (int)((natom + FL_TILE - 1) / FL_TILE);
  const int kgn = std::max<int>(1, (int)((kg.size() + FL_KGRAN - 1) / FL_KGRAN));
  const int a_first = fl_find(f->atom_owner, ag);
  const int k_first = fl_find(f->k_owner, kgn);
  if (a_first < 0 || k_first < 0) {
    yg_set_error("yg_fleet_add: no room left for the system's atoms or k vectors");
    return YG_ERR_CAPACITY;
  }
  FleetSys S;
  std::memset(&S, 0, sizeof(S));
  S.a0 = a_first * FL_TILE;
  S.n = (int)natom;
  S.k0 = k_first * FL_KGRAN;
  S.nk = (int)kg.size();
  S.state = 1;
  S.init = 1;
  for (int k = 0; k < 3; k++) {
    S.rmax[k] = rmax[k];
    S.gmax[k] = gmax[k];
  }
  S.nsteps = (int)nsteps;
  std::memcpy(S.rv, R, sizeof(R));
  std::memcpy(S.gv, G, sizeof(G));
  S.rcut = rcut;
  S.rcs = rcut + skin;
  S.alpha = alpha;
  S.dt = dt;
  S.skin = skin;
  // self energy and neutralizing background (point charges, dielectric 1)
  double q2 = 0.0, qs = 0.0;
  for (int64_t a = 0; a < natom; a++) {
    q2 += charges[a] * charges[a];
    qs += charges[a];
  }
  S.e_const = -alpha / 1.7724538509055160273 * q2 + 3.14159265358979323846 / (2.0 * volume) * qs * qs / alpha / alpha;
  // per-atom arrays
  const int64_t a0 = S.a0;
  std::vector<double> invm(natom);
  std::vector<float> q(natom), sg(natom), se(natom);
  std::vector<int> sid((size_t)ag * FL_TILE, -1);  // the range's padding atoms carry -1: never stepped
  for (int64_t a = 0; a < natom; a++) {
    if (!(masses[a] > 0.0)) return YG_ERR_ARG;
    invm[a] = 1.0 / masses[a];
    q[a] = (float)charges[a];
    sg[a] = (float)sigma[a];
    se[a] = (float)std::sqrt(std::max(epsilon[a], 0.0));
    sid[a] = s;
  }
  // every copy on the fleet's stream, complete before the call returns (the
  // system's id goes in last: it is what makes the kernels step it)
  cudaStream_t st = f->stream;
  const cudaMemcpyKind h2d = cudaMemcpyHostToDevice;
  YG_CUDA(cudaMemcpyAsync(f->d.pos + 3 * a0, pos, natom * 24, h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.pos_build + 3 * a0, pos, natom * 24, h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.vel + 3 * a0, vel, natom * 24, h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.invm + a0, invm.data(), natom * 8, h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.q + a0, q.data(), natom * 4, h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.sig + a0, sg.data(), natom * 4, h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.seps + a0, se.data(), natom * 4, h2d, st));
  YG_CUDA(cudaMemsetAsync(f->d.gtot + 3 * a0, 0, natom * 24, st));
  YG_CUDA(cudaMemsetAsync(f->d.ncount + a0, 0, (size_t)ag * FL_TILE * 4, st));
  YG_CUDA(cudaMemcpyAsync(f->d.kv + S.k0, kv.data(), kv.size() * 16, h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.kslot + S.k0, ksl.data(), ksl.size() * 4, h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.kpref + S.k0, kp.data(), kp.size() * 8, h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.kg + S.k0, kg.data(), kg.size() * 16, h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.d_sys + s, &S, sizeof(S), h2d, st));
  YG_CUDA(cudaMemcpyAsync(f->d.sysid + a0, sid.data(), sid.size() * 4, h2d, st));
  YG_CUDA(cudaStreamSynchronize(st));
  for (int g = 0; g < ag; g++) f->atom_owner[a_first + g] = s;
  for (int g = 0; g < kgn; g++) f->k_owner[k_first + g] = s;
  f->h_sys[s] = S;
  *slot = s;
  return YG_OK;
}

int yg_fleet_remove(yg_fleet *f, int slot) {
  if (!f || slot < 0 || slot >= f->max_systems || f->h_sys[slot].state == 0) return YG_ERR_ARG;
  const FleetSys &S = f->h_sys[slot];
  const int ag = (S.n + FL_TILE - 1) / FL_TILE, kgn = std::max(1, (S.nk + FL_KGRAN - 1) / FL_KGRAN);
  FleetSys z;
  std::memset(&z, 0, sizeof(z));
  YG_CUDA(cudaMemsetAsync(f->d.sysid + S.a0, 0xff, (size_t)ag * FL_TILE * 4, f->stream));
  YG_CUDA(cudaMemsetAsync(f->d.kg + S.k0, 0xff, (size_t)kgn * FL_KGRAN * 16, f->stream));
  YG_CUDA(cudaMemcpyAsync(f->d.d_sys + slot, &z, sizeof(z), cudaMemcpyHostToDevice, f->stream));
  YG_CUDA(cudaStreamSynchronize(f->stream));
  for (auto &o : f->atom_owner)
    if (o == slot) o = -1;
  for (auto &o : f->k_owner)
    if (o == slot) o = -1;
  f->h_sys[slot] = z;
  return YG_OK;
}

int yg_fleet_step(yg_fleet *f, int64_t nsteps) {
  if (!f || nsteps < 0) return YG_ERR_ARG;
  int rc;
  if (!f->graph) {
    // one step captured on a private stream and replayed on the fleet's
    if (!f->cap_stream) YG_CUDA(cudaStreamCreateWithFlags(&f->cap_stream, cudaStreamNonBlocking));
    cudaGraph_t g;
    YG_CUDA(cudaStreamBeginCapture(f->cap_stream, cudaStreamCaptureModeThreadLocal));
    rc = fl_launch_step(f, f->cap_stream);
    cudaGraph_t gg = nullptr;
    cudaError_t e = cudaStreamEndCapture(f->cap_stream, &gg);
    if (rc) return rc;
    if (e != cudaSuccess) return yg_cuda_fail(e, "fleet capture");
    g = gg;
    e = cudaGraphInstantiate(&f->graph, g, 0);
    cudaGraphDestroy(g);
    if (e != cudaSuccess) return yg_cuda_fail(e, "fleet instantiate");
  }
  for (int64_t k = 0; k < nsteps; k++) {
    YG_CUDA(cudaGraphLaunch(f->graph, f->stream));
    f->launches += 8;
  }
  return YG_OK;
}

// States of all slots (0 empty, 1 stepping, 2 done, 3 failed) and the steps
// each has completed; waits for the fleet's stream.
int yg_fleet_poll(yg_fleet *f, int *state, int *steps) {
  if (!f) return YG_ERR_ARG;
  YG_CUDA(cudaMemcpyAsync(f->h_sys_pinned, f->d.d_sys, (size_t)f->max_systems * sizeof(FleetSys),
                          cudaMemcpyDeviceToHost, f->stream));
  YG_CUDA(cudaStreamSynchronize(f->stream));
  for (int s = 0; s < f->max_systems; s++) {
    if (state) state[s] = f->h_sys_pinned[s].state;
    if (steps) steps[s] = f->h_sys_pinned[s].step;
  }
  return YG_OK;
}

int yg_fleet_get(yg_fleet *f, int slot, double *pos, double *vel, double *log, int64_t *nlog) {
  if (!f || slot < 0 || slot >= f->max_systems || f->h_sys[slot].state == 0) return YG_ERR_ARG;
  const FleetSys &S = f->h_sys[slot];
  FleetSys D;
  const cudaMemcpyKind d2h = cudaMemcpyDeviceToHost;
  YG_CUDA(cudaMemcpyAsync(&D, f->d.d_sys + slot, sizeof(D), d2h, f->stream));
  if (pos) YG_CUDA(cudaMemcpyAsync(pos, f->d.pos + 3 * (int64_t)S.a0, (size_t)S.n * 24, d2h, f->stream));
  if (vel) YG_CUDA(cudaMemcpyAsync(vel, f->d.vel + 3 * (int64_t)S.a0, (size_t)S.n * 24, d2h, f->stream));
  YG_CUDA(cudaStreamSynchronize(f->stream));
  const int64_t rows = D.init ? 0 : (int64_t)D.step + 1;
  if (log && rows > 0) {
    YG_CUDA(cudaMemcpyAsync(log, f->d.log + (int64_t)slot * (f->d.max_steps + 1) * 2, (size_t)rows * 16, d2h,
                            f->stream));
    YG_CUDA(cudaStreamSynchronize(f->stream));
  }
  if (nlog) *nlog = rows;
  return D.state == 3 ? YG_ERR_CAPACITY : YG_OK;
}

int yg_fleet_usage(yg_fleet *f, int64_t *atoms_used, int *systems_used, int64_t *k_used) {
  if (!f) return YG_ERR_ARG;
  int64_t a = 0, k = 0;
  int n = 0;
  for (int g : f->atom_owner) a += g >= 0 ? FL_TILE : 0;
  for (int g : f->k_owner) k += g >= 0 ? FL_KGRAN : 0;
  for (const auto &S : f->h_sys) n += S.state != 0;
  if (atoms_used) *atoms_used = a;
  if (systems_used) *systems_used = n;
  if (k_used) *k_used = k;
  return YG_OK;
}

int64_t yg_fleet_launch_count(yg_fleet *f) { return f ? f->launches : -1; }

}  // extern "C"
