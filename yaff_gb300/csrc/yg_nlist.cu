// yg_nlist.cu -- kernel (a): cell-list neighbour build for triclinic cells.
//
// Replaces the O(N^2 * images) scan of yaff/pes/nlist.c:30-131.  Atoms are
// binned on a grid in fractional coordinates whose cells are at least half the
// cutoff wide along every plane normal, counting-sorted by cell (ties by atom
// index, so the order is deterministic), and every atom scans the cells of a
// (2k+1)^3 stencil.  The list is a FULL list (each pair stored from both
// atoms) in per-atom slots, which lets the pair kernel accumulate forces
// without atomics.
//
// Membership is decided exactly as the reference decides it.  Each candidate
// is first tested in FP32 on cell-local coordinates; when the FP32 distance is
// inside or outside the cutoff by more than a guard band (derived from the
// FP32 rounding bound on the host) the decision is final, otherwise the
// reference's own FP64 arithmetic is replayed (sequential minimum-image wrap,
// image shift, squared distance, all with separately rounded multiplies and
// adds) and decides.  The FP32 shortcut is only enabled when the cutoff is
// below half the smallest plane spacing, where the reference can only produce
// central-image rows; otherwise every candidate takes the exact path.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <vector>

#include <mutex>

#include "yg_internal.cuh"

#ifndef YG_CELL_DIV
#define YG_CELL_DIV 4      // grid cells at least r_c / 4 wide
#endif
// Run buffer and candidate map per warp.  Occupancy is bound by registers (4
// blocks of 8 warps per SM at 64 registers), so the smaller buffers (37 KB per
// block instead of 55 KB) leave more of the SM's memory to the L1 cache that
// serves the candidates' coordinates: 0.537 against 0.547 ms per build of the
// 50,000-atom triclinic system.
#ifndef YG_BUILD_RUNS
#define YG_BUILD_RUNS 128  // candidate runs per warp held in shared memory
#endif
#ifndef YG_BUILD_MAP
#define YG_BUILD_MAP 2048  // candidates per warp whose run index is tabulated
#endif

namespace {

__global__ void k_bin(const int *__restrict__ gate, const double *__restrict__ pos, int64_t natom, CellGeom cell, GridGeom grid,
                      int *__restrict__ cell_of, int *__restrict__ wimg, int *__restrict__ count,
                      int *__restrict__ status) {
  if (gate && !*gate) return;
  int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (a >= natom) return;
  double p[3] = {pos[3 * a], pos[3 * a + 1], pos[3 * a + 2]};
  int c[3], w[3];
  bool bad = false;
#pragma unroll
  for (int k = 0; k < 3; k++) {
    double f = cell.gv[3 * k] * p[0] + cell.gv[3 * k + 1] * p[1] + cell.gv[3 * k + 2] * p[2];
    if (!isfinite(f) || fabs(f) > 1e9) {
      bad = true;
      f = 0.0;
    }
    double fl = floor(f);
    double s = f - fl;
    int ci = (int)(s * grid.n[k]);
    if (ci < 0) ci = 0;
    if (ci >= grid.n[k]) ci = grid.n[k] - 1;
    c[k] = ci;
    w[k] = (int)fl;
  }
  if (bad) atomicOr(status + YG_ST_BADCELL, 1);
  int id = c[0] + grid.n[0] * (c[1] + grid.n[1] * c[2]);
  cell_of[a] = id;
  wimg[3 * a] = w[0];
  wimg[3 * a + 1] = w[1];
  wimg[3 * a + 2] = w[2];
  atomicAdd(count + id, 1);
}

// Exclusive scan of the per-cell counts (one block; cell counts are small).
__global__ void k_scan_cells(const int *__restrict__ gate, const int *__restrict__ count, int ncell, int *__restrict__ start,
                             int *__restrict__ fill) {
  if (gate && !*gate) return;
  __shared__ int warp_sums[32];
  __shared__ int carry;
  if (threadIdx.x == 0) carry = 0;
  __syncthreads();
  for (int base = 0; base < ncell; base += blockDim.x) {
    int i = base + threadIdx.x;
    int v = (i < ncell) ? count[i] : 0;
    int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    int x = v;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      int y = __shfl_up_sync(0xffffffffu, x, o);
      if (lane >= o) x += y;
    }
    if (lane == 31) warp_sums[wid] = x;
    __syncthreads();
    if (wid == 0) {
      int nw = blockDim.x >> 5;
      int s = (lane < nw) ? warp_sums[lane] : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        int y = __shfl_up_sync(0xffffffffu, s, o);
        if (lane >= o) s += y;
      }
      if (lane < nw) warp_sums[lane] = s;
    }
    __syncthreads();
    int excl = x - v + (wid > 0 ? warp_sums[wid - 1] : 0) + carry;
    if (i < ncell) {
      start[i] = excl;
      fill[i] = excl;
    }
    __syncthreads();
    if (threadIdx.x == blockDim.x - 1) carry = excl + v;
    __syncthreads();
  }
  if (threadIdx.x == 0) start[ncell] = carry;
}

__global__ void k_scatter(const int *__restrict__ gate, const int *__restrict__ cell_of, int64_t natom, int *__restrict__ fill,
                          int *__restrict__ sorted) {
  if (gate && !*gate) return;
  int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (a >= natom) return;
  int slot = atomicAdd(fill + cell_of[a], 1);
  sorted[slot] = (int)a;
}

// Orders the atoms of every cell by index.  One warp per cell: each lane
// holds up to 4 entries and computes their ranks by comparing with all
// entries of the cell through shuffles (indices are distinct), then writes
// them to their final slots.  Cells with more than 128 atoms (pathological
// densities) fall back to an insertion sort by lane 0.
__global__ void k_sort_cells(const int *__restrict__ gate, const int *__restrict__ start, int ncell, int *__restrict__ sorted) {
  if (gate && !*gate) return;
  const int c = (int)((blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5);
  const int lane = threadIdx.x & 31;
  if (c >= ncell) return;
  const int s0 = start[c], s1 = start[c + 1];
  const int n = s1 - s0;
  if (n <= 1) return;
  if (n > 128) {
    if (lane == 0) {
      for (int i = s0 + 1; i < s1; i++) {
        int v = sorted[i];
        int j = i - 1;
        while (j >= s0 && sorted[j] > v) {
          sorted[j + 1] = sorted[j];
          j--;
        }
        sorted[j + 1] = v;
      }
    }
    return;
  }
  int v[4], rank[4];
#pragma unroll
  for (int q = 0; q < 4; q++) {
    v[q] = (lane + 32 * q < n) ? sorted[s0 + lane + 32 * q] : 0x7fffffff;
    rank[q] = 0;
  }
  for (int src = 0; src < n; src++) {
    const int qs = src >> 5;
    const int mine = qs == 0 ? v[0] : (qs == 1 ? v[1] : (qs == 2 ? v[2] : v[3]));
    const int w = __shfl_sync(0xffffffffu, mine, src & 31);
#pragma unroll
    for (int q = 0; q < 4; q++) rank[q] += (w < v[q]) ? 1 : 0;
  }
  __syncwarp();
#pragma unroll
  for (int q = 0; q < 4; q++)
    if (lane + 32 * q < n) sorted[s0 + rank[q]] = v[q];
}

// Cell origin (FP64) of every sorted atom and the orig -> sorted map.
__global__ void k_origins(const int *__restrict__ gate, const int *__restrict__ sorted, const int *__restrict__ cell_of,
                          const int *__restrict__ wimg, int64_t natom, CellGeom cell, GridGeom grid,
                          const double *__restrict__ cfrac, double *__restrict__ org, int *__restrict__ rank) {
  if (gate && !*gate) return;
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= natom) return;
  int a = sorted[s];
  int id = cell_of[a];
  int c[3] = {id % grid.n[0], (id / grid.n[0]) % grid.n[1], id / (grid.n[0] * grid.n[1])};
  double f[3];
  // c / n from the host table (the same IEEE quotient, without FP64 divisions here)
#pragma unroll
  for (int k = 0; k < 3; k++) f[k] = (double)wimg[3 * a + k] + cfrac[512 * k + c[k]];
#pragma unroll
  for (int x = 0; x < 3; x++)
    org[3 * s + x] = f[0] * cell.rv[x] + f[1] * cell.rv[3 + x] + f[2] * cell.rv[6 + x];
  rank[a] = (int)s;
}

// Per-evaluation refresh of the cell-local coordinates (FP64 and FP32) and
// charges in sorted order.  Cell assignment stays frozen between rebuilds.
__global__ void k_prep(const double *__restrict__ pos, const double *__restrict__ charge,
                       const int *__restrict__ sorted, const double *__restrict__ org, const int *__restrict__ cell_of,
                       int ncx, int64_t natom, double4_32a *__restrict__ x64, float4 *__restrict__ x32,
                       float4 *__restrict__ xb) {
  int64_t s = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (s >= natom) return;
  int a = sorted[s];
  double q = charge ? charge[a] : 0.0;
  double x = pos[3 * a] - org[3 * s];
  double y = pos[3 * a + 1] - org[3 * s + 1];
  double z = pos[3 * a + 2] - org[3 * s + 2];
  x64[s] = make_double4_32a(x, y, z, q);
  x32[s] = make_float4((float)x, (float)y, (float)z, (float)q);
  // build coordinates: the 4th lane carries the cell's x index
  xb[s] = make_float4((float)x, (float)y, (float)z, __int_as_float(cell_of[a] % ncx));
}

// floor(u / n) for the cell offsets of the sweep: u = home cell + stencil
// offset, so when the stencil half-width k is at most n the quotient is -1, 0
// or 1 (two compares instead of an integer division by a run-time n).
__device__ __forceinline__ int floordiv_near(int u, int n, bool near) {
  if (near) return (u < 0) ? -1 : (u >= n ? 1 : 0);
  int q = u / n;
  if (u < 0 && q * n != u) q--;
  return q;
}

__device__ __forceinline__ int floordiv(int u, int n) {
  int q = u / n;
  if (u < 0 && q * n != u) q--;
  return q;
}

__device__ __forceinline__ int excl_code(const int *__restrict__ estart, const int2 *__restrict__ excl,
                                         int oi, int oj) {
  if (!estart) return 0;
  int s0 = estart[oi], s1 = estart[oi + 1];
  for (int e = s0; e < s1; e++) {
    int2 v = excl[e];
    if (v.x == oj) return v.y;
  }
  return 0;
}

struct BuildArgs {
  CellGeom cell;
  GridGeom grid;
  const double *pos;
  const int *sorted;
  const int *cell_of;
  const int *wimg;
  const int *cell_start;
  const float4 *x32;
  const float4 *xb;       // build coordinates, w = cell x index
  const float4 *shift32;
  const int *estart;
  const int2 *excl;
  uint2 *nbr;
  int2 *ncount;     // (front, back) entry counts of every row
  int *status;
  unsigned long long *total;
  int64_t natom;
  int64_t cap;
  int64_t nlow, nhigh;
  int rmax[3];
  double rc2;
  float lo, hi;     // FP32 guard band on d^2
  float rin2;       // FP32 d^2 below which an entry goes to the row's front
                    // (the pair cutoff squared, with a margin above the
                    // rounding of either precision's d)
  int fast;
  int filter;       // nlow/nhigh restrict the pairs
  const int *gate;  // device flag: build only when set (nullptr: always)
  const int4 *rows; // pruned stencil rows (o1, o2, lo, hi)
  float pm[9], pw[3], pg[9], pg0[3], pkeep;  // per-atom row trimming (see trim_row)
};

// The x-offset interval of stencil row (o1, o2, lo, hi) that can hold
// candidates of an atom at (phi0, phi1, phi2) of its home cell (cell widths
// along each axis, from the cell's corner): trimmed from both ends while the
// cell at the end is provably beyond the list's reach.  The bound for the
// cell at offset o: along the direction u to its centre p = sum_k c_k M_k
// (c_k = o_k - phi_k + 1/2, M_k its edge vectors), every point d of the cell
// has |d| >= u.d >= |p| - sum_k |u.M_k| / 2.  Along a row only c_0 changes,
// so q = c_1 M_1 + c_2 M_2 and its products are formed once per row and a
// cell costs |p|^2 = c_0^2 M_0.M_0 + 2 c_0 M_0.q + q.q and
// p.M_k = c_0 M_0.M_k + q.M_k.  A row whose slab bound along axis 1 or 2
// (w_k times the gap to the row) already reaches the limit is empty.  Cells
// inside the interval are kept, so every cell holding a neighbour stays.
__device__ __forceinline__ int2 trim_row(const BuildArgs &A, int4 row, float phi0, float phi1, float phi2) {
  const float a1 = (float)row.x - phi1, a2 = (float)row.y - phi2;
  if (A.pw[1] * fmaxf(0.f, fmaxf(a1, -a1 - 1.f)) >= A.pkeep || A.pw[2] * fmaxf(0.f, fmaxf(a2, -a2 - 1.f)) >= A.pkeep)
    return make_int2(1, 0);
  const float c1 = a1 + 0.5f, c2 = a2 + 0.5f;
  const float qx = c1 * A.pm[3] + c2 * A.pm[6], qy = c1 * A.pm[4] + c2 * A.pm[7], qz = c1 * A.pm[5] + c2 * A.pm[8];
  const float qq = qx * qx + qy * qy + qz * qz;
  const float qm0 = qx * A.pm[0] + qy * A.pm[1] + qz * A.pm[2];
  const float qm1 = qx * A.pm[3] + qy * A.pm[4] + qz * A.pm[5];
  const float qm2 = qx * A.pm[6] + qy * A.pm[7] + qz * A.pm[8];
  auto beyond = [&](int o0) {
    const float c0 = (float)o0 - phi0 + 0.5f;
    const float pp = fmaf(c0, fmaf(c0, A.pg0[0], 2.0f * qm0), qq);
    const float ext = fabsf(fmaf(c0, A.pg0[0], qm0)) + fabsf(fmaf(c0, A.pg0[1], qm1)) + fabsf(fmaf(c0, A.pg0[2], qm2));
    if (!(pp > 0.f)) return false;
    const float inv = rsqrtf(pp);
    return pp * inv - 0.5f * inv * ext >= A.pkeep;
  };
  int lo = row.z, hi = row.w;
  while (lo <= hi && beyond(lo)) lo++;
  while (hi >= lo && beyond(hi)) hi--;
  return make_int2(lo, hi);
}

// Exact replay of the reference's decision for candidate (oi -> oj) whose
// image relative to the raw position difference is t (pos_j - pos_i + t.R).
// Returns 1 when the pair is in the list; *central is set when its image is 0.
__device__ __forceinline__ int exact_decide(const BuildArgs &A, int oi, int oj, const int *t,
                                            int *central) {
  *central = 0;
  int r[3];
  double d[3];
  if (oi == oj) {
    // self image: the wrapped relative vector is zero, the image is t
    for (int k = 0; k < 3; k++) r[k] = t[k];
    if (img_zero(r)) return 0;
    if (!img_positive(r)) for (int k = 0; k < 3; k++) r[k] = -r[k];
    for (int k = 0; k < 3; k++)
      if (r[k] > A.rmax[k] || r[k] < -A.rmax[k]) return 0;
    d[0] = 0.0; d[1] = 0.0; d[2] = 0.0;
    exact_add_vec(d, A.cell, r);
    return exact_norm2(d) < A.rc2;
  }
  int a = max(oi, oj), b = min(oi, oj);
  int tab[3];
  for (int k = 0; k < 3; k++) tab[k] = (oi == a) ? t[k] : -t[k];
  d[0] = xsub(A.pos[3 * b], A.pos[3 * a]);
  d[1] = xsub(A.pos[3 * b + 1], A.pos[3 * a + 1]);
  d[2] = xsub(A.pos[3 * b + 2], A.pos[3 * a + 2]);
  int m[3];
  exact_mic(d, A.cell, m);
  for (int k = 0; k < 3; k++) {
    r[k] = tab[k] + m[k];
    if (r[k] > A.rmax[k] || r[k] < -A.rmax[k]) return 0;
  }
  if (img_zero(r)) {
    *central = 1;
  } else if (!img_positive(r)) {
    for (int k = 0; k < 3; k++) {
      r[k] = -r[k];
      d[k] = -d[k];
    }
  }
  exact_add_vec(d, A.cell, r);
  return exact_norm2(d) < A.rc2;
}

#define YG_RUN_MAX 8   // cells per contiguous x run of the stencil
// The candidate sweep loads the next chunk's candidate and coordinates while
// the current chunk is tested (0.565 against 0.612 ms per build of the
// 50,000-atom triclinic system); 0 selects the plain loop.
#ifndef YG_BUILD_PIPELINE
#define YG_BUILD_PIPELINE 1
#endif

// One warp per sorted atom.  Every (o1, o2) row of the stencil is swept as
// runs of x-consecutive cells that share one periodic image; the atoms of a
// run are contiguous in sorted order, so lanes walk them in full 32-wide
// chunks and recover each candidate's x offset from the cell boundaries of
// the run (kept in registers).
// One candidate run: atoms s0 .. s0+len-1 (contiguous in sorted order: one
// to several x-consecutive cells of one stencil row sharing one periodic
// image), oidx = obase + cell x of the candidate, packed images and the
// home-row flag.
__device__ __forceinline__ int pack_img(int n0, int n1, int n2, int home) {
  return (n0 + 512) | ((n1 + 512) << 10) | ((n2 + 512) << 20) | (home << 30);
}

// One warp per sorted atom.  The candidates of all stencil rows of a batch
// are laid out as runs in shared memory (lanes build the runs of different
// rows in parallel), then swept as one flat index space 32 at a time, so
// short runs of the fine grid do not leave lanes idle.
// Dynamic shared memory of k_build per warp: runs, run offsets, candidate map.
#define YG_BUILD_WARP_SMEM (YG_BUILD_RUNS * 16 + (YG_BUILD_RUNS + 4) * 4 + YG_BUILD_MAP)
// the map area doubles as the trimmed-row buffer of a batch (at most 96
// int2) and every warp's area stays 8-byte aligned
#define YG_BUILD_ROWCAP 96
static_assert(YG_BUILD_MAP >= YG_BUILD_ROWCAP * 8 && YG_BUILD_MAP % 8 == 0 && YG_BUILD_RUNS % 2 == 0,
              "build buffers: map of at least 768 bytes, 8-byte multiples");

#ifndef YG_BUILD_MINB
#define YG_BUILD_MINB 4  // resident blocks per SM of the candidate sweep
#endif
__global__ void __launch_bounds__(256, YG_BUILD_MINB) k_build(BuildArgs A) {
  extern __shared__ __align__(16) unsigned char build_smem[];
  if (A.gate && !*A.gate) return;
  int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  const int lane = threadIdx.x & 31, wv = threadIdx.x >> 5;
  if (i >= A.natom) return;
  unsigned char *wsm = build_smem + (size_t)wv * YG_BUILD_WARP_SMEM;
  int4 *run = reinterpret_cast<int4 *>(wsm);
  int *off = reinterpret_cast<int *>(wsm + YG_BUILD_RUNS * 16);
  unsigned char *map = wsm + YG_BUILD_RUNS * 16 + (YG_BUILD_RUNS + 4) * 4;  // run of every candidate of the batch
  const int oi = A.sorted[i];
  const float4 xi = A.x32[i];
  const int cid = A.cell_of[oi];
  // the atom's place in its cell (xi is relative to the cell's corner)
  const float phi0 = A.pg[0] * xi.x + A.pg[1] * xi.y + A.pg[2] * xi.z;
  const float phi1 = A.pg[3] * xi.x + A.pg[4] * xi.y + A.pg[5] * xi.z;
  const float phi2 = A.pg[6] * xi.x + A.pg[7] * xi.y + A.pg[8] * xi.z;
  const int N0 = A.grid.n[0], N1 = A.grid.n[1], N2 = A.grid.n[2];
  const int ci[3] = {cid % N0, (cid / N0) % N1, cid / (N0 * N1)};
  const int wi[3] = {A.wimg[3 * oi], A.wimg[3 * oi + 1], A.wimg[3 * oi + 2]};
  const bool need_oj = A.filter || A.estart != nullptr || !A.fast;
  int64_t base = 0, back = 0;  // entries at the row's front and back
  int nexact = 0;
  uint2 *out = A.nbr + i * A.cap;
  const int K0 = A.grid.k[0], K1 = A.grid.k[1], K2 = A.grid.k[2];
  const bool near0 = K0 <= N0, near1 = K1 <= N1, near2 = K2 <= N2;
  const int w0 = 2 * K0 + 1, w1 = 2 * K1 + 1;
  const int oidx_home = K0 + w0 * (K1 + w1 * K2);
  for (int rb = 0; rb < A.grid.nrow; rb += A.grid.rows_per_batch) {
    const int re = min(A.grid.nrow, rb + A.grid.rows_per_batch);
    // runs per lane: count, warp scan, then write; each row trimmed to the
    // atom's reach, the trimmed interval kept in the (still idle) map area
    // for the writing pass (a batch holds at most YG_BUILD_ROWCAP rows)
    int2 *trim = reinterpret_cast<int2 *>(map);
    int mine = 0;
    for (int r = rb + lane; r < re; r += 32) {
      const int2 t = trim_row(A, A.rows[r], phi0, phi1, phi2);
      trim[r - rb] = t;
      for (int ox = t.x; ox <= t.y;) {
        const int u0 = ci[0] + ox;
        const int c0 = u0 - floordiv_near(u0, N0, near0) * N0;
        ox += min(t.y - ox + 1, N0 - c0);
        mine++;
      }
    }
    int incl = mine;
#pragma unroll
    for (int o = 1; o < 32; o <<= 1) {
      const int y = __shfl_up_sync(0xffffffffu, incl, o);
      if (lane >= o) incl += y;
    }
    const int nrun = __shfl_sync(0xffffffffu, incl, 31);
    int slot = incl - mine;
    for (int r = rb + lane; r < re; r += 32) {
      const int2 t = trim[r - rb];
      if (t.x > t.y) continue;
      const int4 row = make_int4(A.rows[r].x, A.rows[r].y, t.x, t.y);
      const int o1 = row.x, o2 = row.y;
      const int u1 = ci[1] + o1, u2 = ci[2] + o2;
      const int n1 = floordiv_near(u1, N1, near1), n2 = floordiv_near(u2, N2, near2);
      const int c1 = u1 - n1 * N1, c2 = u2 - n2 * N2;
      const int rowcell = N0 * (c1 + N1 * c2);
      const int orow = w0 * ((o1 + K1) + w1 * (o2 + K2));
      for (int ox = row.z; ox <= row.w;) {
        const int u0 = ci[0] + ox;
        const int n0 = floordiv_near(u0, N0, near0);
        const int c0 = u0 - n0 * N0;
        const int len = min(row.w - ox + 1, N0 - c0);
        const int s0 = A.cell_start[rowcell + c0], s1 = A.cell_start[rowcell + c0 + len];
        run[slot] = make_int4(s0, s1 - s0, ox - c0 + K0 + orow,
                              pack_img(n0, n1, n2, (o1 == 0 && o2 == 0 && n0 == 0) ? 1 : 0));
        slot++;
        ox += len;
      }
    }
    __syncwarp();
    // candidate offsets of the runs
    int carry = 0;
    for (int b = 0; b < nrun; b += 32) {
      int v = (b + lane < nrun) ? run[b + lane].y : 0;
#pragma unroll
      for (int o = 1; o < 32; o <<= 1) {
        const int y = __shfl_up_sync(0xffffffffu, v, o);
        if (lane >= o) v += y;
      }
      if (b + lane < nrun) off[b + lane + 1] = carry + v;
      carry += __shfl_sync(0xffffffffu, v, 31);
    }
    if (lane == 0) off[0] = 0;
    __syncwarp();
    const int total = carry;
    // a batch whose candidates fit the map gets each candidate's run written
    // once (lanes fill the runs' ranges), so the sweep looks it up instead of
    // stepping through the run offsets
    const bool mapped = total <= YG_BUILD_MAP && nrun <= 256;
    // a run's start becomes relative to the flat candidate index (candidate
    // q of run b is atom run[b].x + q)
    for (int b = lane; b < nrun; b += 32) {
      const int o = off[b];
      run[b].x -= o;
      if (mapped) {
        const int c1 = off[b + 1];
        for (int c = o; c < c1; c++) map[c] = (unsigned char)b;
      }
    }
    __syncwarp();
    int r = 0;
    if (mapped && A.fast && !need_oj) {
      // common case (no exclusions, no nlow/nhigh filter, FP32 shortcut on):
      // branch-free FP32 test, the exact replay only for the rare candidates
      // inside the guard band; 32-bit row positions
      const int cap32 = (int)min(A.cap, (int64_t)0x7fffffff);
      int base32 = (int)base, back32 = (int)back;
      const unsigned lt = (1u << lane) - 1u;
#if YG_BUILD_PIPELINE
      // the next chunk's candidate and coordinates are loaded while this
      // chunk is tested (one load chain in flight ahead)
      int qn = min(lane, total - 1);
      int rqn = map[qn];
      int4 rrn = run[rqn];
      int jn = rrn.x + qn;
      float4 xjn = A.xb[jn];
      for (int q0 = 0; q0 < total; q0 += 32) {
        const bool live = q0 + lane < total;
        const int4 rr = rrn;
        const int j = jn;
        const float4 xj = xjn;
        if (q0 + 32 < total) {
          qn = min(q0 + 32 + lane, total - 1);
          rqn = map[qn];
          rrn = run[rqn];
          jn = rrn.x + qn;
          xjn = A.xb[jn];
        }
#else
      for (int q0 = 0; q0 < total; q0 += 32) {
        const int q = min(q0 + lane, total - 1);
        const bool live = q0 + lane < total;
        const int rq = map[q];
        const int4 rr = run[rq];
        const int j = rr.x + q;
        const float4 xj = A.xb[j];
#endif
        const int oidx = rr.z + __float_as_int(xj.w);
        const float4 sh = A.shift32[oidx];
        const float dx = (xj.x - xi.x) + sh.x;
        const float dy = (xj.y - xi.y) + sh.y;
        const float dz = (xj.z - xi.z) + sh.z;
        const float d2 = dx * dx + dy * dy + dz * dz;
        const bool self0 = (rr.w >> 30) && (j == i) && (oidx == oidx_home);
        const bool ok = live && !self0;
        int in = (ok && d2 < A.lo) ? 1 : 0;
        int central = 1;
        if (ok && d2 >= A.lo && d2 <= A.hi) {
          const int oj = A.sorted[j];
          const int pk = rr.w;
          const int n0 = (pk & 1023) - 512, n1 = ((pk >> 10) & 1023) - 512, n2 = ((pk >> 20) & 1023) - 512;
          int tt[3] = {n0 + wi[0] - A.wimg[3 * oj], n1 + wi[1] - A.wimg[3 * oj + 1], n2 + wi[2] - A.wimg[3 * oj + 2]};
          in = exact_decide(A, oi, oj, tt, &central);
          nexact++;
        }
        const bool front = d2 < A.rin2;
        const unsigned bf = __ballot_sync(0xffffffffu, in && front);
        const unsigned bb = __ballot_sync(0xffffffffu, in && !front);
        if (in) {
          const int pos = front ? base32 + __popc(bf & lt) : back32 + __popc(bb & lt);
          if (pos < cap32)
            out[front ? pos : cap32 - 1 - pos] =
                make_uint2((unsigned)j, (unsigned)oidx | (central ? YG_META_CENTRAL : 0u));
        }
        base32 += __popc(bf);
        back32 += __popc(bb);
      }
      base = base32;
      back = back32;
    }
    for (int q0 = (mapped && A.fast && !need_oj) ? total : 0; q0 < total; q0 += 32) {
      const int q = q0 + lane;
      int in = 0, central = 1, oj = -1, oidx = 0, j = 0;
      bool front = false;
      if (q < total) {
        if (mapped) r = map[q];
        else
          while (off[r + 1] <= q) r++;
        const int4 rr = run[r];
        j = rr.x + q;
        const float4 xj = A.xb[j];
        oidx = rr.z + __float_as_int(xj.w);
        const int pk = rr.w;
        const bool self0 = (pk >> 30) && (j == i) && (oidx == oidx_home);
        bool keep = !self0;
        if (keep && need_oj) {
          oj = A.sorted[j];
          if (A.filter) {
            const int a = max(oi, oj), b = min(oi, oj);
            keep = (a >= A.nlow && b < A.nhigh) || (b >= A.nlow && a < A.nhigh);
          }
        }
        if (keep) {
          const float4 sh = A.shift32[oidx];
          const float dx = (xj.x - xi.x) + sh.x;
          const float dy = (xj.y - xi.y) + sh.y;
          const float dz = (xj.z - xi.z) + sh.z;
          const float d2 = dx * dx + dy * dy + dz * dz;
          front = d2 < A.rin2;
          int decided = 0;
          if (A.fast) {
            if (d2 < A.lo) { in = 1; decided = 1; }
            else if (d2 > A.hi) { in = 0; decided = 1; }
          }
          if (!decided) {
            if (oj < 0) oj = A.sorted[j];
            const int n0 = (pk & 1023) - 512, n1 = ((pk >> 10) & 1023) - 512, n2 = ((pk >> 20) & 1023) - 512;
            int tt[3] = {n0 + wi[0] - A.wimg[3 * oj], n1 + wi[1] - A.wimg[3 * oj + 1],
                         n2 + wi[2] - A.wimg[3 * oj + 2]};
            in = exact_decide(A, oi, oj, tt, &central);
            nexact++;
          }
        }
      }
      const unsigned bf = __ballot_sync(0xffffffffu, in && front);
      const unsigned bb = __ballot_sync(0xffffffffu, in && !front);
      if (in) {
        const int code = (central && A.estart) ? excl_code(A.estart, A.excl, oi, oj) : 0;
        const unsigned lt = (1u << lane) - 1u;
        const int64_t p = front ? base + __popc(bf & lt) : back + __popc(bb & lt);
        if (p < A.cap) {
          const unsigned meta = (unsigned)oidx | ((unsigned)code << YG_META_SCALE_SHIFT) |
                                (central ? YG_META_CENTRAL : 0u);
          out[front ? p : A.cap - 1 - p] = make_uint2((unsigned)j, meta);
        }
      }
      base += __popc(bf);
      back += __popc(bb);
    }
    __syncwarp();  // the next batch overwrites this warp's runs
  }
  for (int o = 16; o > 0; o >>= 1) nexact += __shfl_down_sync(0xffffffffu, nexact, o);
  if (lane == 0) {
    // an overflowing row keeps disjoint segments (its entries are discarded)
    const int64_t nf = min(base, A.cap), nb = min(back, A.cap - nf), all = base + back;
    A.ncount[i] = make_int2((int)nf, (int)nb);
    if (all > A.cap) atomicOr(A.status + YG_ST_OVERFLOW, 1);
    atomicMax(A.status + YG_ST_MAXCOUNT, (int)min(all, (int64_t)0x7fffffff));
    if (nexact) atomicAdd(A.status + YG_ST_EXACT, nexact);
    atomicAdd(A.total, (unsigned long long)(nf + nb));
  }
}

struct ExportArgs {
  BuildArgs B;
  const double *pos_now;
  int recomputed;
  yg_neigh_row *rows;
  unsigned long long *nrows;
  int64_t cap_rows;
};

// Emits every reference row once, from the entry whose atom is the row's
// larger index (self images: from the entry with the positive image).
__global__ void k_export(ExportArgs E) {
  const BuildArgs &A = E.B;
  int64_t i = (blockIdx.x * (int64_t)blockDim.x + threadIdx.x) >> 5;
  int lane = threadIdx.x & 31;
  if (i >= A.natom) return;
  const int oi = A.sorted[i];
  const int cid = A.cell_of[oi];
  const int ci[3] = {cid % A.grid.n[0], (cid / A.grid.n[0]) % A.grid.n[1], cid / (A.grid.n[0] * A.grid.n[1])};
  const int wi[3] = {A.wimg[3 * oi], A.wimg[3 * oi + 1], A.wimg[3 * oi + 2]};
  const int2 cn = A.ncount[i];
  const int w0 = 2 * A.grid.k[0] + 1, w1 = 2 * A.grid.k[1] + 1;
  for (int e = lane; e < cn.x + cn.y; e += 32) {
    uint2 ent = A.nbr[i * A.cap + (e < cn.x ? e : A.cap - cn.y + (e - cn.x))];
    int j = (int)ent.x;
    int oidx = (int)(ent.y & YG_META_OFF_MASK);
    int o0 = oidx % w0 - A.grid.k[0];
    int o1 = (oidx / w0) % w1 - A.grid.k[1];
    int o2 = oidx / (w0 * w1) - A.grid.k[2];
    int u[3] = {ci[0] + o0, ci[1] + o1, ci[2] + o2};
    int nimg[3];
    for (int k = 0; k < 3; k++) nimg[k] = floordiv(u[k], A.grid.n[k]);
    int oj = A.sorted[j];
    int t[3] = {nimg[0] + wi[0] - A.wimg[3 * oj], nimg[1] + wi[1] - A.wimg[3 * oj + 1],
                nimg[2] + wi[2] - A.wimg[3 * oj + 2]};
    int ra, rb, r[3];
    double d[3];
    if (oi == oj) {
      if (!img_positive(t)) continue;
      for (int k = 0; k < 3; k++) r[k] = t[k];
      ra = oi; rb = oi;
      d[0] = 0.0; d[1] = 0.0; d[2] = 0.0;
    } else {
      if (oi < oj) continue;
      int a = oi, b = oj;
      d[0] = xsub(A.pos[3 * b], A.pos[3 * a]);
      d[1] = xsub(A.pos[3 * b + 1], A.pos[3 * a + 1]);
      d[2] = xsub(A.pos[3 * b + 2], A.pos[3 * a + 2]);
      int m[3];
      exact_mic(d, A.cell, m);
      for (int k = 0; k < 3; k++) r[k] = t[k] + m[k];
      ra = a; rb = b;
      if (!img_zero(r) && !img_positive(r)) {
        for (int k = 0; k < 3; k++) {
          r[k] = -r[k];
          d[k] = -d[k];
        }
        ra = b; rb = a;
      }
    }
    if (E.recomputed) {
      // skin path of the reference: image from the old (build) positions,
      // relative vector from the current ones (yaff/pes/nlist.c:183-232)
      double o[3] = {xsub(A.pos[3 * rb], A.pos[3 * ra]), xsub(A.pos[3 * rb + 1], A.pos[3 * ra + 1]),
                     xsub(A.pos[3 * rb + 2], A.pos[3 * ra + 2])};
      int ctr[3];
      exact_to_center(o, A.cell, ctr);
      d[0] = xsub(E.pos_now[3 * rb], E.pos_now[3 * ra]);
      d[1] = xsub(E.pos_now[3 * rb + 1], E.pos_now[3 * ra + 1]);
      d[2] = xsub(E.pos_now[3 * rb + 2], E.pos_now[3 * ra + 2]);
      exact_add_vec(d, A.cell, ctr);
    }
    exact_add_vec(d, A.cell, r);
    double dd = exact_norm2(d);
    unsigned long long slot = atomicAdd(E.nrows, 1ull);
    if ((int64_t)slot < E.cap_rows) {
      yg_neigh_row row;
      row.a = ra;
      row.b = rb;
      row.d = __dsqrt_rn(dd);
      row.dx = d[0];
      row.dy = d[1];
      row.dz = d[2];
      row.r0 = r[0];
      row.r1 = r[1];
      row.r2 = r[2];
      E.rows[slot] = row;
    }
  }
}

__global__ void k_max_disp2(const double *__restrict__ pos, const double *__restrict__ old, int64_t natom,
                            unsigned long long *__restrict__ out) {
  double m = 0.0;
  for (int64_t a = blockIdx.x * (int64_t)blockDim.x + threadIdx.x; a < natom;
       a += (int64_t)gridDim.x * blockDim.x) {
    double dx = pos[3 * a] - old[3 * a];
    double dy = pos[3 * a + 1] - old[3 * a + 1];
    double dz = pos[3 * a + 2] - old[3 * a + 2];
    double v = dx * dx + dy * dy + dz * dz;
    if (!(v <= m)) m = v;   // also propagates NaN
  }
  for (int o = 16; o > 0; o >>= 1) m = fmax(m, __shfl_down_sync(0xffffffffu, m, o));
  if ((threadIdx.x & 31) == 0) atomicMax(out, (unsigned long long)__double_as_longlong(m));
}

// Repacks the per-atom pair parameters into sorted order:
// for every potential p: sigma, sqrt(epsilon), radius^2, onlypauli.
__global__ void k_pack_params(const int *__restrict__ gate, const double *__restrict__ src, const int *__restrict__ sorted, int64_t natom,
                              double *__restrict__ dst64, float *__restrict__ dst32) {
  if (gate && !*gate) return;
  // one thread per (sorted atom, value): coalesced stores
  const int64_t idx = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  if (idx >= natom * 4 * YG_MAX_POT) return;
  const int64_t s = idx / (4 * YG_MAX_POT);
  const int v = (int)(idx - s * (4 * YG_MAX_POT));
  const double x = src[(int64_t)sorted[s] * 4 * YG_MAX_POT + v];
  dst64[idx] = x;
  dst32[idx] = (float)x;
}

// The row split of a build: the largest cutoff of the registered pair
// potentials (the list cutoff when there is none).  The sweep compares its
// FP32 d^2 with rin^2 (1 + 2e-5): the FP32 d^2 and the d of either pair
// kernel differ by far less, so no entry within a pair cutoff lands in the
// back segment.
double pair_split(const yg_ctx *ctx) {
  double rin = 0.0;
  for (int p = 0; p < YG_MAX_POT; p++)
    if (ctx->pot[p].active && ctx->pot[p].rcut > rin) rin = ctx->pot[p].rcut;
  if (!(rin > 0.0) || rin > ctx->rcut_total) rin = ctx->rcut_total;
  return rin;
}

BuildArgs make_args(yg_ctx *ctx, double rc2) {
  BuildArgs A;
  A.cell = ctx->cell;
  A.grid = ctx->grid;
  A.pos = ctx->d_pos_build;
  A.sorted = ctx->d_sorted;
  A.cell_of = ctx->d_cell_of;
  A.wimg = ctx->d_wimg;
  A.cell_start = ctx->d_cell_start;
  A.x32 = ctx->d_x32;
  A.xb = ctx->d_xb;
  A.shift32 = ctx->d_shift32;
  A.estart = ctx->nexcl ? ctx->d_excl_start : nullptr;
  A.excl = ctx->d_excl;
  A.nbr = ctx->d_nbr;
  A.ncount = ctx->d_ncount;
  A.status = ctx->d_status;
  A.total = nullptr;
  A.natom = ctx->natom;
  A.cap = ctx->nbr_cap;
  A.nlow = ctx->nlow;
  A.nhigh = ctx->nhigh;
  for (int k = 0; k < 3; k++) A.rmax[k] = (int)ctx->rmax[k];
  A.rc2 = rc2;
  A.lo = 0.0f;
  A.hi = 0.0f;
  {
    const double rin = pair_split(ctx);
    A.rin2 = (float)(rin * rin * (1.0 + 2e-5));
  }
  A.fast = 0;
  A.filter = (ctx->nlow > 0 || ctx->nhigh < ctx->natom) ? 1 : 0;
  A.gate = nullptr;
  A.rows = ctx->d_rows;
  for (int k = 0; k < 9; k++) {
    A.pm[k] = ctx->prune_pm[k];
    A.pg[k] = ctx->prune_pg[k];
  }
  for (int k = 0; k < 3; k++) {
    A.pw[k] = ctx->prune_pw[k];
    A.pg0[k] = ctx->prune_g0[k];
  }
  A.pkeep = ctx->prune_keep;
  return A;
}

}  // namespace

// Uploads the pair parameters of all potentials (orig order) when they
// changed, then repacks them into sorted order on the device.
int yg_pack_pair_params(yg_ctx *ctx) {
  size_t n = (size_t)ctx->natom * 4 * YG_MAX_POT;
  int rc;
  if (!ctx->d_pp64) {
    if ((rc = yg_alloc(ctx, (void **)&ctx->d_pp_src, n * sizeof(double)))) return rc;
    if ((rc = yg_alloc(ctx, (void **)&ctx->d_pp64, n * sizeof(double)))) return rc;
    if ((rc = yg_alloc(ctx, (void **)&ctx->d_pp32, n * sizeof(float)))) return rc;
    ctx->pp_dirty = 1;
  }
  if (ctx->pp_dirty) {
    std::vector<double> h(n, 0.0);
    for (int p = 0; p < YG_MAX_POT; p++) {
      const PairPotHost &P = ctx->pot[p];
      if (!P.active) continue;
      for (int64_t a = 0; a < ctx->natom; a++) {
        double *q = h.data() + (size_t)a * 4 * YG_MAX_POT + 4 * p;
        q[0] = !P.types.empty() ? (double)P.types[a] : P.sigma.empty() ? 0.0 : P.sigma[a];
        q[1] = P.sqrteps.empty() ? 0.0 : P.sqrteps[a];
        q[2] = P.radius2.empty() ? 0.0 : P.radius2[a];
        q[3] = P.onlypauli.empty() ? 0.0 : (double)P.onlypauli[a];
      }
    }
    YG_CUDA(cudaMemcpyAsync(ctx->d_pp_src, h.data(), n * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    ctx->pp_dirty = 0;
  }
  k_pack_params<<<yg_blocks(ctx->natom * 4 * YG_MAX_POT, 256), 256, 0, ctx->stream>>>(nullptr, ctx->d_pp_src, ctx->d_sorted, ctx->natom,
                                                                     ctx->d_pp64, ctx->d_pp32);
  YG_LAUNCH_CHECK(ctx, "k_pack_params");
  ctx->pp_packed = 1;
  return YG_OK;
}

int yg_launch_prep_positions(yg_ctx *ctx) {
  k_prep<<<yg_blocks(ctx->natom, 256), 256, 0, ctx->stream>>>(
      ctx->d_pos, ctx->have_charges ? ctx->d_charge : nullptr, ctx->d_sorted, ctx->d_org, ctx->d_cell_of,
      ctx->grid.n[0], ctx->natom, ctx->d_x64, ctx->d_x32, ctx->d_xb);
  YG_LAUNCH_CHECK(ctx, "k_prep");
  ctx->x_fresh = 0;  // the rows no longer match the coordinates (a host build sets it again)
  return YG_OK;
}

// Largest squared displacement since the last rebuild, as the bits of a
// non-negative double, max-combined into *out (which the caller zeroes).
int yg_launch_max_disp2_async(yg_ctx *ctx, unsigned long long *out) {
  k_max_disp2<<<yg_blocks(ctx->natom, 256) > 1024 ? 1024 : yg_blocks(ctx->natom, 256), 256, 0, ctx->stream>>>(
      ctx->d_pos, ctx->d_pos_build, ctx->natom, out);
  YG_LAUNCH_CHECK(ctx, "k_max_disp2");
  return YG_OK;
}

int yg_launch_max_disp2(yg_ctx *ctx, double *out) {
  unsigned long long *d = (unsigned long long *)ctx->d_red;
  YG_CUDA(cudaMemsetAsync(d, 0, sizeof(unsigned long long), ctx->stream));
  k_max_disp2<<<yg_blocks(ctx->natom, 256) > 1024 ? 1024 : yg_blocks(ctx->natom, 256), 256, 0, ctx->stream>>>(
      ctx->d_pos, ctx->d_pos_build, ctx->natom, d);
  YG_LAUNCH_CHECK(ctx, "k_max_disp2");
  unsigned long long h = 0;
  YG_CUDA(cudaMemcpyAsync(&h, d, sizeof(h), cudaMemcpyDeviceToHost, ctx->stream));
  YG_CUDA(cudaStreamSynchronize(ctx->stream));
  double v;
  memcpy(&v, &h, sizeof(v));
  *out = v;
  return YG_OK;
}

// Host-side geometry of a build for the current cell and cutoff: the cell
// grid, the stencil shift vectors (uploaded) and the FP32 guard band.  Kept
// until the cell or the cutoff changes.
static int nlist_geometry(yg_ctx *ctx, double rc2) {
  const double rc = ctx->rcut_total;
  if (ctx->geom_valid && ctx->geom_rc == rc) return YG_OK;
  const CellGeom &C = ctx->cell;
  // grid: cells at least rc/YG_CELL_DIV wide along each plane normal
  GridGeom G;
  double rsp[3];
  for (int k = 0; k < 3; k++) {
    const double *g = C.gv + 3 * k;
    rsp[k] = 1.0 / std::sqrt(g[0] * g[0] + g[1] * g[1] + g[2] * g[2]);
    int n = (int)std::floor(rsp[k] / (rc / YG_CELL_DIV));
    if (n < 1) n = 1;
    if (n > 512) n = 512;
    G.n[k] = n;
    double w = rsp[k] / n;
    double rsearch = rc * (1.0 + 1e-9) + 1e-9;
    G.k[k] = (int)std::ceil(rsearch / w);
  }
  G.noff = (2 * G.k[0] + 1) * (2 * G.k[1] + 1) * (2 * G.k[2] + 1);
  G.ncell = G.n[0] * G.n[1] * G.n[2];
  if (G.noff > 65535) {
    yg_set_error("neighbour stencil too large for this cutoff/cell combination");
    return YG_ERR_UNSUPPORTED;
  }
  int rc_ = YG_OK;
  if (G.ncell + 1 > ctx->cap_sorted) {
    yg_free(ctx, (void **)&ctx->d_cell_start);
    yg_free(ctx, (void **)&ctx->d_cell_fill);
    if ((rc_ = yg_alloc(ctx, (void **)&ctx->d_cell_start, (G.ncell + 1) * sizeof(int)))) return rc_;
    if ((rc_ = yg_alloc(ctx, (void **)&ctx->d_cell_fill, (G.ncell + 1) * sizeof(int)))) return rc_;
    ctx->cap_sorted = G.ncell + 1;
  }
  ctx->grid = G;
  // shift vectors of the stencil
  std::vector<double> sh64(3 * (size_t)G.noff);
  std::vector<float4> sh32(G.noff);
  double maxsh = 0.0;
  for (int o2 = -G.k[2]; o2 <= G.k[2]; o2++)
    for (int o1 = -G.k[1]; o1 <= G.k[1]; o1++)
      for (int o0 = -G.k[0]; o0 <= G.k[0]; o0++) {
        int idx = (o0 + G.k[0]) + (2 * G.k[0] + 1) * ((o1 + G.k[1]) + (2 * G.k[1] + 1) * (o2 + G.k[2]));
        double f[3] = {(double)o0 / G.n[0], (double)o1 / G.n[1], (double)o2 / G.n[2]};
        double v[3];
        for (int x = 0; x < 3; x++) v[x] = f[0] * C.rv[x] + f[1] * C.rv[3 + x] + f[2] * C.rv[6 + x];
        for (int x = 0; x < 3; x++) sh64[3 * idx + x] = v[x];
        sh32[idx] = make_float4((float)v[0], (float)v[1], (float)v[2], 0.0f);
        maxsh = std::max(maxsh, std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
      }
  // stencil rows that can hold neighbours, each with the interval of x offsets
  // whose cells can lie within the cutoff: a cell pair at offset o is at
  // least max_u (u.M o - sum_k |u.M_k|) apart (M_k = cell edge vectors; any
  // unit u gives a lower bound), tried for u along M (o + clamp(-o)) and M o,
  // and the slab bounds (|o_k| - 1) h_k along the plane normals
  std::vector<int4> rows;
  {
    double Mk[3][3];  // Mk[k] = rv_k / n_k
    for (int k = 0; k < 3; k++)
      for (int x = 0; x < 3; x++) Mk[k][x] = C.rv[3 * k + x] / G.n[k];
    const double keep_below = rc * (1.0 + 1e-6) + 1e-6;
    auto lower_bound = [&](const int o[3]) {
      double lb = 0.0;
      for (int k = 0; k < 3; k++) lb = std::max(lb, (std::abs(o[k]) - 1.0) * rsp[k] / G.n[k]);
      double mo[3], mt[3];
      for (int x = 0; x < 3; x++) {
        mo[x] = 0.0;
        mt[x] = 0.0;
        for (int k = 0; k < 3; k++) {
          const double t = std::min(1.0, std::max(-1.0, (double)-o[k]));
          mo[x] += o[k] * Mk[k][x];
          mt[x] += (o[k] + t) * Mk[k][x];
        }
      }
      for (const double *p : {mt, mo}) {
        const double nrm = std::sqrt(p[0] * p[0] + p[1] * p[1] + p[2] * p[2]);
        if (!(nrm > 0.0)) continue;
        const double u[3] = {p[0] / nrm, p[1] / nrm, p[2] / nrm};
        double v = u[0] * mo[0] + u[1] * mo[1] + u[2] * mo[2];
        for (int k = 0; k < 3; k++) v -= std::abs(u[0] * Mk[k][0] + u[1] * Mk[k][1] + u[2] * Mk[k][2]);
        lb = std::max(lb, v);
      }
      return lb;
    };
    for (int o2 = -G.k[2]; o2 <= G.k[2]; o2++)
      for (int o1 = -G.k[1]; o1 <= G.k[1]; o1++) {
        int lo = G.k[0] + 1, hi = -G.k[0] - 1;
        for (int o0 = -G.k[0]; o0 <= G.k[0]; o0++) {
          const int o[3] = {o0, o1, o2};
          if (lower_bound(o) < keep_below) {
            lo = std::min(lo, o0);
            hi = std::max(hi, o0);
          }
        }
        if (lo <= hi) rows.push_back(make_int4(o1, o2, lo, hi));
      }
  }
  G.nrow = (int)rows.size();
  {
    const int maxruns = (2 * G.k[0] + 1 + G.n[0] - 1) / G.n[0] + 1;  // x wraps split a row
    G.rows_per_batch = std::min(YG_BUILD_ROWCAP, std::max(1, YG_BUILD_RUNS / maxruns));  // trimmed-row buffer
    if (maxruns > YG_BUILD_RUNS) {
      yg_set_error("neighbour stencil row too long for the build kernel");
      return YG_ERR_UNSUPPORTED;
    }
  }
  ctx->grid = G;
  // grow-only: buffers keep their addresses across rebuilds (captured graphs
  // refer to them)
  if ((rc_ = yg_ensure(ctx, (void **)&ctx->d_rows, &ctx->rows_cap, std::max<size_t>(1, rows.size()) * sizeof(int4))))
    return rc_;
  if (!rows.empty())
    YG_CUDA(cudaMemcpyAsync(ctx->d_rows, rows.data(), rows.size() * sizeof(int4), cudaMemcpyHostToDevice, ctx->stream));
  if ((rc_ = yg_ensure(ctx, (void **)&ctx->d_shift64, &ctx->shift64_cap, sh64.size() * sizeof(double)))) return rc_;
  if ((rc_ = yg_ensure(ctx, (void **)&ctx->d_shift32, &ctx->shift32_cap, sh32.size() * sizeof(float4)))) return rc_;
  YG_CUDA(cudaMemcpyAsync(ctx->d_shift64, sh64.data(), sh64.size() * sizeof(double), cudaMemcpyHostToDevice, ctx->stream));
  YG_CUDA(cudaMemcpyAsync(ctx->d_shift32, sh32.data(), sh32.size() * sizeof(float4), cudaMemcpyHostToDevice, ctx->stream));
  // c / n_k for every grid index (n_k <= 512)
  std::vector<double> cfrac(3 * 512, 0.0);
  for (int k = 0; k < 3; k++)
    for (int c = 0; c < G.n[k]; c++) cfrac[512 * k + c] = (double)c / (double)G.n[k];
  if (!ctx->d_cfrac && (rc_ = yg_alloc(ctx, (void **)&ctx->d_cfrac, cfrac.size() * sizeof(double)))) return rc_;
  YG_CUDA(cudaMemcpyAsync(ctx->d_cfrac, cfrac.data(), cfrac.size() * sizeof(double), cudaMemcpyHostToDevice,
                          ctx->stream));
  YG_CUDA(cudaStreamSynchronize(ctx->stream));  // the host vectors go out of scope

  // FP32 guard band: bound on |d2_fp32 - d2_exact| from the magnitudes of the
  // cell-local coordinates (< one cell diagonal) and the shift vectors.
  double celldiag = 0.0;
  {
    double f[3] = {1.0 / G.n[0], 1.0 / G.n[1], 1.0 / G.n[2]};
    for (int s0 = -1; s0 <= 1; s0 += 2)
      for (int s1 = -1; s1 <= 1; s1 += 2) {
        double v[3];
        for (int x = 0; x < 3; x++) v[x] = f[0] * C.rv[x] + s0 * f[1] * C.rv[3 + x] + s1 * f[2] * C.rv[6 + x];
        celldiag = std::max(celldiag, std::sqrt(v[0] * v[0] + v[1] * v[1] + v[2] * v[2]));
      }
    celldiag *= 1.01;
  }
  double eps32 = 5.960464477539063e-08;  // 2^-24
  double comp = 8.0 * eps32 * (maxsh + 2.0 * celldiag + rc);
  double err = 2.0 * rc * std::sqrt(3.0) * comp + 3.0 * comp * comp + 4.0 * eps32 * rc2;
  err *= 4.0;  // safety factor
  double min_half = 0.5 * std::min(rsp[0], std::min(rsp[1], rsp[2]));
  ctx->fast_path = (rc * (1.0 + 1e-7) + 1e-7 < min_half) ? 1 : 0;
  float lo = (float)(rc2 - err), hi = (float)(rc2 + err);
  // make the band closed under FP32 rounding of the thresholds themselves
  ctx->band_lo = nextafterf(nextafterf(lo, 0.0f), 0.0f);
  ctx->band_hi = nextafterf(nextafterf(hi, INFINITY), INFINITY);
  // per-atom row trimming: a cell whose lower-bound distance from the atom
  // reaches prune_keep (above the guard band by 1e-5 relative + 1e-3 bohr,
  // far beyond the FP32 rounding of the bound) holds no candidate that could
  // enter the list
  for (int k = 0; k < 3; k++) {
    ctx->prune_pw[k] = (float)(rsp[k] / G.n[k]);
    for (int x = 0; x < 3; x++) {
      ctx->prune_pm[3 * k + x] = (float)(C.rv[3 * k + x] / G.n[k]);
      ctx->prune_pg[3 * k + x] = (float)(C.gv[3 * k + x] * G.n[k]);
    }
  }
  for (int k = 0; k < 3; k++)
    ctx->prune_g0[k] = (float)((C.rv[0] * C.rv[3 * k] + C.rv[1] * C.rv[3 * k + 1] + C.rv[2] * C.rv[3 * k + 2]) /
                               ((double)G.n[0] * G.n[k]));  // M_0 . M_k
  ctx->prune_keep = (float)(std::sqrt((double)ctx->band_hi) * (1.0 + 1e-5) + 1e-3);

  // neighbour slots
  if (ctx->nbr_cap == 0) {
    double dens = ctx->natom / C.volume;
    double est = dens * 4.18879020478639 * rc * rc * rc;  // 4/3 pi rc^3
    int64_t cap = (int64_t)(est * 1.3) + 64;
    cap = (cap + 31) / 32 * 32;
    ctx->nbr_cap = cap;
  }
  ctx->geom_rc = rc;
  ctx->geom_valid = 1;
  return YG_OK;
}

__global__ void k_build_reset(const int *__restrict__ gate, int *__restrict__ cell_fill, int ncell1,
                              const double *__restrict__ pos, double *__restrict__ pos_build, int64_t n3,
                              unsigned long long *__restrict__ total) {
  if (gate && !*gate) return;
  const int64_t stride = (int64_t)gridDim.x * blockDim.x;
  const int64_t t0 = blockIdx.x * (int64_t)blockDim.x + threadIdx.x;
  for (int64_t t = t0; t < ncell1; t += stride) cell_fill[t] = 0;
  for (int64_t t = t0; t < n3; t += stride) pos_build[t] = pos[t];
  if (t0 == 0) *total = 0ull;
}

// Enqueues one build for the current positions (no host synchronization):
// reset, bin, counting sort, origins, cell-local coordinates, candidate
// sweep.  With a gate, every kernel returns at once unless *gate is set.
static int enqueue_build(yg_ctx *ctx, double rc2, const int *gate, unsigned long long *total) {
  const int64_t N = ctx->natom;
  const CellGeom &C = ctx->cell;
  const GridGeom &G = ctx->grid;
  const int64_t n3 = N * 3;
  const int64_t big = std::max<int64_t>(n3, G.ncell + 1);
  k_build_reset<<<(int)std::min<int64_t>(yg_blocks(big, 256), 1024), 256, 0, ctx->stream>>>(
      gate, ctx->d_cell_fill, G.ncell + 1, ctx->d_pos, ctx->d_pos_build, n3, total);
  YG_LAUNCH_CHECK(ctx, "k_build_reset");
  k_bin<<<yg_blocks(N, 256), 256, 0, ctx->stream>>>(gate, ctx->d_pos, N, C, G, ctx->d_cell_of, ctx->d_wimg,
                                                    ctx->d_cell_fill, ctx->d_status);
  YG_LAUNCH_CHECK(ctx, "k_bin");
  k_scan_cells<<<1, 1024, 0, ctx->stream>>>(gate, ctx->d_cell_fill, G.ncell, ctx->d_cell_start, ctx->d_cell_fill);
  YG_LAUNCH_CHECK(ctx, "k_scan_cells");
  k_scatter<<<yg_blocks(N, 256), 256, 0, ctx->stream>>>(gate, ctx->d_cell_of, N, ctx->d_cell_fill, ctx->d_sorted);
  YG_LAUNCH_CHECK(ctx, "k_scatter");
  k_sort_cells<<<yg_blocks((int64_t)G.ncell * 32, 256), 256, 0, ctx->stream>>>(gate, ctx->d_cell_start, G.ncell,
                                                                                ctx->d_sorted);
  YG_LAUNCH_CHECK(ctx, "k_sort_cells");
  k_origins<<<yg_blocks(N, 256), 256, 0, ctx->stream>>>(gate, ctx->d_sorted, ctx->d_cell_of, ctx->d_wimg, N, C, G,
                                                        ctx->d_cfrac, ctx->d_org, ctx->d_rank);
  YG_LAUNCH_CHECK(ctx, "k_origins");
  int rc_;
  if ((rc_ = yg_launch_prep_positions(ctx))) return rc_;
  BuildArgs A = make_args(ctx, rc2);
  A.fast = ctx->fast_path;
  A.lo = ctx->band_lo;
  A.hi = ctx->band_hi;
  A.total = total;
  A.gate = gate;
  const size_t bsm = (size_t)8 * YG_BUILD_WARP_SMEM;
  static int optin_dev = -1;  // the dynamic shared-memory limit is raised once per device
  {
    static std::mutex mu;
    int dev = 0;
    YG_CUDA(cudaGetDevice(&dev));
    std::lock_guard<std::mutex> lk(mu);
    if (optin_dev != dev) {
      YG_CUDA(cudaFuncSetAttribute((const void *)k_build, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bsm));
      optin_dev = dev;
    }
  }
  k_build<<<yg_blocks(N * 32, 256), 256, bsm, ctx->stream>>>(A);
  YG_LAUNCH_CHECK(ctx, "k_build");
  return YG_OK;
}

int yg_launch_nlist_build(yg_ctx *ctx, double rc2, int *retry) {
  int rc_;
  if ((rc_ = nlist_geometry(ctx, rc2))) return rc_;
  const int64_t N = ctx->natom;
  for (;;) {
    int64_t need = ctx->nbr_cap * N;
    if (need > ctx->nbr_alloc) {
      yg_free(ctx, (void **)&ctx->d_nbr);
      if ((rc_ = yg_alloc(ctx, (void **)&ctx->d_nbr, (size_t)need * sizeof(uint2)))) return rc_;
      ctx->nbr_alloc = need;
    }
    unsigned long long *dtot = (unsigned long long *)ctx->d_red;
    YG_CUDA(cudaMemsetAsync(ctx->d_status, 0, YG_ST_NWORDS * sizeof(int), ctx->stream));
    if ((rc_ = enqueue_build(ctx, rc2, nullptr, dtot))) return rc_;
    YG_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->d_status, YG_ST_NWORDS * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
    unsigned long long *htot = ctx->h_u64;
    YG_CUDA(cudaMemcpyAsync(htot, dtot, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
    YG_CUDA(cudaStreamSynchronize(ctx->stream));
    if (ctx->h_status[YG_ST_BADCELL]) {
      yg_set_error("non-finite or huge position met while binning atoms");
      return YG_ERR_NAN;
    }
    if (ctx->h_status[YG_ST_OVERFLOW]) {
      int64_t cap = (int64_t)(ctx->h_status[YG_ST_MAXCOUNT] * 1.15) + 64;
      ctx->nbr_cap = (cap + 31) / 32 * 32;
      if (retry) (*retry)++;
      continue;
    }
    ctx->nneigh = (int64_t)(*htot / 2);
    break;
  }
  ctx->have_list = 1;
  ctx->rows_valid = 1;
  ctx->list_recomputed = 0;
  ctx->rin_build = pair_split(ctx);
  ctx->x_fresh = 1;
  // the sorted order changed: repack the pair parameters
  if ((rc_ = yg_pack_pair_params(ctx))) return rc_;
  return YG_OK;
}

// One build enqueued without waiting: its status words and pair count are
// copied to the page-locked mirrors behind it and ctx->build_ev marks their
// arrival; the pair parameters are repacked behind it too.  The rows are used
// at once (the pair terms are enqueued after the build on the same stream);
// yg_nlist_build_wait reports an overflow or a bad position before any result
// that used them is read.
int yg_launch_nlist_build_async(yg_ctx *ctx, double rc2) {
  int rc_;
  if ((rc_ = nlist_geometry(ctx, rc2))) return rc_;
  const int64_t need = ctx->nbr_cap * ctx->natom;
  if (need > ctx->nbr_alloc) {
    yg_free(ctx, (void **)&ctx->d_nbr);
    if ((rc_ = yg_alloc(ctx, (void **)&ctx->d_nbr, (size_t)need * sizeof(uint2)))) return rc_;
    ctx->nbr_alloc = need;
  }
  unsigned long long *dtot = (unsigned long long *)ctx->d_red;
  YG_CUDA(cudaMemsetAsync(ctx->d_status, 0, YG_ST_NWORDS * sizeof(int), ctx->stream));
  if ((rc_ = enqueue_build(ctx, rc2, nullptr, dtot))) return rc_;
  YG_CUDA(cudaMemcpyAsync(ctx->h_status, ctx->d_status, YG_ST_NWORDS * sizeof(int), cudaMemcpyDeviceToHost, ctx->stream));
  YG_CUDA(cudaMemcpyAsync(ctx->h_u64 + 6, dtot, sizeof(unsigned long long), cudaMemcpyDeviceToHost, ctx->stream));
  if (!ctx->build_ev) YG_CUDA(cudaEventCreateWithFlags(&ctx->build_ev, cudaEventDisableTiming));
  YG_CUDA(cudaEventRecord(ctx->build_ev, ctx->stream));
  ctx->build_pending = 1;
  ctx->have_list = 1;
  ctx->rows_valid = 1;
  ctx->list_recomputed = 0;
  ctx->rin_build = pair_split(ctx);
  ctx->x_fresh = 1;
  return yg_pack_pair_params(ctx);
}

// Waits for an enqueued build's status.  YG_OK: ctx->nneigh holds its pair
// count.  YG_ERR_CAPACITY: a row overflowed; the slot capacity is grown and
// the rows are invalid until the next build (results computed from them must
// be recomputed).  YG_ERR_NAN: a position could not be binned.
int yg_launch_nlist_build_wait(yg_ctx *ctx) {
  if (!ctx->build_pending) return YG_OK;
  ctx->build_pending = 0;
  YG_CUDA(cudaEventSynchronize(ctx->build_ev));
  if (ctx->h_status[YG_ST_BADCELL]) {
    ctx->rows_valid = 0;
    yg_set_error("non-finite or huge position met while binning atoms");
    return YG_ERR_NAN;
  }
  if (ctx->h_status[YG_ST_OVERFLOW]) {
    const int64_t cap = (int64_t)(ctx->h_status[YG_ST_MAXCOUNT] * 1.15) + 64;
    ctx->nbr_cap = (cap + 31) / 32 * 32;
    ctx->rows_valid = 0;
    yg_set_error("a neighbour row overflowed its slots; rebuild the list and recompute");
    return YG_ERR_CAPACITY;
  }
  ctx->nneigh = (int64_t)(ctx->h_u64[6] / 2);
  return YG_OK;
}

// A rebuild that runs only when *gate is set, for the device-driven step:
// no host synchronization; overflow and bad positions accumulate in the
// status words (cleared by the caller), the pair count goes to *total.
int yg_launch_nlist_build_gated(yg_ctx *ctx, const int *gate, unsigned long long *total) {
  int rc_;
  if (!ctx->geom_valid || !ctx->have_list) {
    yg_set_error("gated rebuild needs a host build first");
    return YG_ERR_STATE;
  }
  const double rc2 = ctx->rcut_total * ctx->rcut_total;
  if ((rc_ = enqueue_build(ctx, rc2, gate, total))) return rc_;
  ctx->rin_build = pair_split(ctx);
  k_pack_params<<<yg_blocks(ctx->natom * 4 * YG_MAX_POT, 256), 256, 0, ctx->stream>>>(gate, ctx->d_pp_src, ctx->d_sorted, ctx->natom,
                                                                     ctx->d_pp64, ctx->d_pp32);
  YG_LAUNCH_CHECK(ctx, "k_pack_params");
  return YG_OK;
}

int yg_launch_nlist_export(yg_ctx *ctx, yg_neigh_row *rows_host, int64_t cap, int64_t *n) {
  int64_t want = ctx->nneigh;
  *n = want;
  if (want > cap || rows_host == nullptr) return YG_OK;
  yg_neigh_row *d_rows = nullptr;
  int rc = yg_alloc(ctx, (void **)&d_rows, (size_t)(want > 0 ? want : 1) * sizeof(yg_neigh_row));
  if (rc) return rc;
  unsigned long long *dcount = (unsigned long long *)ctx->d_red;
  YG_CUDA(cudaMemsetAsync(dcount, 0, sizeof(unsigned long long), ctx->stream));
  ExportArgs E;
  E.B = make_args(ctx, ctx->rcut_total * ctx->rcut_total);
  E.pos_now = ctx->d_pos;
  E.recomputed = ctx->list_recomputed;
  E.rows = d_rows;
  E.nrows = dcount;
  E.cap_rows = want;
  k_export<<<yg_blocks(ctx->natom * 32, 256), 256, 0, ctx->stream>>>(E);
  YG_LAUNCH_CHECK(ctx, "k_export");
  unsigned long long got = 0;
  YG_CUDA(cudaMemcpyAsync(&got, dcount, sizeof(got), cudaMemcpyDeviceToHost, ctx->stream));
  YG_CUDA(cudaMemcpyAsync(rows_host, d_rows, (size_t)want * sizeof(yg_neigh_row), cudaMemcpyDeviceToHost, ctx->stream));
  YG_CUDA(cudaStreamSynchronize(ctx->stream));
  yg_free(ctx, (void **)&d_rows);
  if ((int64_t)got != want) {
    yg_set_error("neighbour export row count differs from the build count");
    return YG_ERR_STATE;
  }
  std::sort(rows_host, rows_host + want, [](const yg_neigh_row &x, const yg_neigh_row &y) {
    if (x.a != y.a) return x.a < y.a;
    if (x.b != y.b) return x.b < y.b;
    if (x.r0 != y.r0) return x.r0 < y.r0;
    if (x.r1 != y.r1) return x.r1 < y.r1;
    return x.r2 < y.r2;
  });
  return YG_OK;
}
