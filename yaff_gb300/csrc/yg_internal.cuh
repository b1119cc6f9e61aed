// yg_internal.cuh -- shared definitions of the GB300 force-evaluation library.
//
// Device state of one system lives in yg_ctx.  Atoms are kept in two orders:
// "orig" (the caller's indexing, used for every input and output array) and
// "sorted" (binned by neighbour-list cell, used by the hot kernels so that the
// atoms of one cell are contiguous in memory).
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>
#include <string>
#include <unordered_map>
#include <vector>

#include "../../include/yaffgb.h"

#define YG_MAX_POT 3
#define YG_RB_CHUNKS 4   // chunks of the pipelined gradient readback
#ifndef YG_FORCE_PAIRS
#define YG_FORCE_PAIRS 1  // tcgen05 Ewald force pass over conjugate column pairs (P formed once per pair)
#endif
#define YG_WARP 32

// Device status words (yg_ctx::d_status)
#define YG_ST_OVERFLOW 0     // a neighbour row did not fit its per-atom slot
#define YG_ST_MAXCOUNT 1     // largest per-atom full-list row count seen
#define YG_ST_EXACT 2        // candidates decided by the exact FP64 test
#define YG_ST_BADCELL 3      // non-finite position met while binning
#define YG_ST_TIMEOUT 4      // a bounded wait on an asynchronous copy gave up
#define YG_ST_NANGRAD 5      // a summed gradient component was NaN (yg_get_total)
#define YG_ST_NWORDS 8

// Neighbour entry: x = partner (sorted index), y = meta bits.
#define YG_META_OFF_MASK 0xFFFFu     // stencil offset index
#define YG_META_SCALE_SHIFT 16       // 3-bit scaling code (0 = none, 1..4 = nbond)
#define YG_META_CENTRAL (1u << 19)   // image r == 0 (scalings apply)

struct CellGeom {
  double rv[9];   // cell vectors (rows)
  double gv[9];   // reciprocal vectors (rows), inv(rv)^T
  double volume;
  int nvec;
};

// Geometry of the cell-list grid used by the neighbour build.
struct GridGeom {
  int n[3];        // cells per axis
  int k[3];        // stencil half width per axis
  int noff;        // (2k0+1)(2k1+1)(2k2+1)
  int ncell;
  int nrow;        // stencil rows (o1, o2) that can hold neighbours
  int rows_per_batch;  // rows whose runs fit the build kernel's run buffer
};

struct PairPotHost {
  int active = 0;
  int kind = 0;
  int tr_kind = 0;
  double rcut = 0.0;
  double tr_par = 0.0;
  double alpha = 0.0;
  double dielectric = 1.0;
  std::vector<double> sigma, sqrteps, radius2;
  std::vector<int32_t> onlypauli;
  // type-pair table kinds: per-atom type, per type pair (a, b, c, d)
  int ntype = 0;
  int power = 0;
  std::vector<int32_t> types;
  std::vector<double> table;
};

// Parameters of one pair potential as the pair kernel sees them.
struct PairPotDev {
  int kind;
  int tr_kind;
  double rcut;
  double rcut2;
  double tr_par;
  double alpha;
  double inv_diel;
  int has_radii;
  int col;        // parameter column (= result slot) of this potential
  int ntype;      // type-pair table kinds: number of atom types
  int power;      // DampDisp: power of 1/d
  const double4_32a *tab64;  // ntype*ntype entries (FP64)
  const float4 *tab32;       // same, FP32
};

// Resident-block count of a kernel at a dynamic shared-memory size (cached).
struct yg_occ {
  const void *fn = nullptr;
  size_t smem = 0;
  int blocks = 0;  // resident blocks per SM x SMs
};

struct yg_ctx {
  int64_t natom = 0;
  int nsm = 1;                    // streaming multiprocessors of the context's device
  int precision = YG_FP64;
  cudaStream_t stream = 0;
  cudaMemPool_t pool = nullptr;   // stream-ordered pool of this context's device
  void *h_block = nullptr;        // pinned host block holding h_status and h_total
  size_t h_block_bytes = 0;
  std::unordered_map<void *, size_t> alloc_bytes;  // live device buffers
  int64_t bytes_now = 0, bytes_high = 0;
  int64_t alloc_calls = 0;
  int64_t launches = 0;

  CellGeom cell{};
  int have_cell = 0;
  int have_pos = 0;

  // positions and charges (orig order)
  double *d_pos = nullptr;        // natom*3 current
  double *d_pos_build = nullptr;  // natom*3 at the last rebuild
  double *d_charge = nullptr;     // natom
  std::vector<double> h_charge;   // host copy (Ewald self term)
  double h_qmax = 0.0, h_qsum = 0.0;  // max |q| and sum |q| of h_charge
  int have_charges = 0;

  // binning (orig order)
  int *d_cell_of = nullptr;       // natom
  int *d_wimg = nullptr;          // natom*3 integer wrap of the fractional coordinates
  // sorted order
  int *d_sorted = nullptr;        // sorted -> orig
  int *d_rank = nullptr;          // orig -> sorted
  int *d_cell_start = nullptr;    // ncell+1
  int *d_cell_fill = nullptr;     // ncell (scratch for the counting sort)
  double *d_org = nullptr;        // sorted*3 cell origin of each atom (FP64)
  double4_32a *d_x64 = nullptr;       // sorted: local coordinate (x,y,z) and charge
  float4 *d_x32 = nullptr;        // sorted: same in FP32
  float4 *d_xb = nullptr;         // sorted: FP32 coordinates, w = cell x index (build)
  int4 *d_rows = nullptr;         // stencil rows (o1, o2, lo, hi) of the pruned stencil
  size_t rows_cap = 0;
  double *d_shift64 = nullptr;    // noff*3 stencil shift vectors
  float4 *d_shift32 = nullptr;    // noff
  size_t shift64_cap = 0, shift32_cap = 0;
  double *d_cfrac = nullptr;      // 3 x 512: c / n_k of every grid index (IEEE division, on the host)
  int cap_sorted = 0;             // allocated cell-list capacity (cells)
  GridGeom grid{};
  int have_list = 0;
  int rows_valid = 0;             // the slot rows hold the current list (cleared by yg_nlist_set_capacity)
  int list_recomputed = 0;        // skin path ran since the last rebuild
  int fast_path = 0;
  int geom_valid = 0;             // grid, shifts and band match (cell, geom_rc)
  double geom_rc = 0.0;
  float band_lo = 0.0f, band_hi = 0.0f;  // FP32 guard band on d^2
  // per-atom trimming of the stencil rows in the candidate sweep: cell edge
  // vectors M_k = rv_k / n_k, slab widths along the plane normals, n_k g_k
  // (cell widths per unit of cell-local position), M_0 . M_k, and the
  // distance beyond which a cell holds no candidate of the list (above the
  // guard band)
  float prune_pm[9] = {0}, prune_pw[3] = {0}, prune_pg[9] = {0}, prune_g0[3] = {0}, prune_keep = 0.0f;
  double rcut_total = 0.0;
  int64_t rmax[3] = {0, 0, 0};
  int64_t nlow = 0, nhigh = 0;
  int64_t nneigh = 0;

  // full neighbour list: per sorted atom a slot of `nbr_cap` entries; the
  // entries within the pair cutoff (rin_build) fill the slot from the front,
  // those of the skin shell from the back: d_ncount = (front, back) counts
  uint2 *d_nbr = nullptr;
  int2 *d_ncount = nullptr;
  double rin_build = 0.0;         // the pair cutoff that split the last build's rows
  int x_fresh = 0;                // the cell-local coordinates are those of the last host build
  const int *pair_fresh_dev = nullptr;  // while capturing the MD step: device flag "rebuilt this step"
  int64_t nbr_cap = 0;
  int64_t nbr_alloc = 0;          // entries allocated
  int *d_status = nullptr;        // YG_ST_NWORDS
  int *h_status = nullptr;        // pinned mirror
  unsigned long long *h_u64 = nullptr;  // pinned: 8 words for small readbacks

  // exclusions: per-atom CSR over orig indices, both directions
  int *d_excl_start = nullptr;    // natom+1
  int2 *d_excl = nullptr;         // (partner, nbond)
  int64_t nexcl = 0;
  double scale_tab[5] = {1.0, 1.0, 1.0, 1.0, 1.0};
  // the scaling table itself (for the Ewald correction)
  int64_t nstab = 0;
  int2 *d_stab_ab = nullptr;
  double *d_stab_scale = nullptr;

  // pair potentials
  PairPotHost pot[YG_MAX_POT];
  double *d_pp_src = nullptr;     // orig*4*YG_MAX_POT: sigma, sqrt(eps), radius^2, onlypauli
  double *d_pp64 = nullptr;       // same in sorted order
  float *d_pp32 = nullptr;        // same, FP32
  double4_32a *d_ptab64[YG_MAX_POT] = {nullptr, nullptr, nullptr};  // type-pair tables per slot
  float4 *d_ptab32[YG_MAX_POT] = {nullptr, nullptr, nullptr};
  int pp_dirty = 1;
  int pp_packed = 0;

  // Ewald
  int have_ewald = 0;
  double ew_alpha = 0.0, ew_gcut = 0.0, ew_diel = 1.0;
  int64_t ew_gmax[3] = {0, 0, 0};
  int64_t ew_nlow = 0, ew_nhigh = 0;
  int ew_ncol = 0;                // (2G0+1)(2G1+1)
  int ew_nm = 0;                  // G2+1
  int ew_nk = 0;                  // k vectors in the half sphere
  double *d_ew_pref = nullptr;    // ncol*nm prefactor (0 outside the half sphere)
  int *d_ew_tiles = nullptr;      // column tiles: (g0 base, g1 base, m_hi)
  int *d_ew_pcols = nullptr;      // conjugate column pairs of the tensor-core S pass: per tile 64 '+' then 64 partners
  int ew_ntp = 0;                 // tiles of 64 pairs
  int *d_ew_uslot = nullptr;      // slot of every dense column in the tcgen05 force pass's tile list (-1: none)
  int ew_ntile = 0;
  int ew_nftile = 0;              // force tiles (EW_FC columns) with work
  int *d_ew_wslot = nullptr;      // dense column -> slot in the tiled weights
  void *d_ew_tab = nullptr;       // per-atom phase tables (complex, T)
  void *d_ew_Spart = nullptr;     // partial structure factors
  double *d_ew_S = nullptr;       // 3 groups * ncol*nm complex (re, im)
  void *d_ew_W = nullptr;         // weights for the force pass, per group
  double *d_ew_gpart = nullptr;   // force partials
  double *d_ew_red = nullptr;     // energy/virial partials of the reciprocal sum
  size_t ew_red_cap = 0;
  // the reciprocal sum runs on its own stream, forked from the context's
  // stream at launch and joined back before its inputs change or its
  // results are read
  cudaStream_t ew_aux = nullptr;
  cudaEvent_t ew_fork_ev = nullptr, ew_join_ev = nullptr;
  int ew_pending = 0;
  size_t ew_bytes_tab = 0, ew_bytes_Spart = 0, ew_bytes_W = 0, ew_bytes_gpart = 0;
  // tensor-core (warp MMA) form of the mixed-precision reciprocal sum
  int ew_mma = 0;                 // 1 when the k-space layout suits it (G2 + 1 <= 32)
  double ew_amax = 0.0;           // largest prefactor A(k)
  int ew_nft4 = 0;                // 4-column force tiles with work
  int ew_wbunits = 0;             // 1 KB fragment units of one group's weights
  int *d_ew_woff = nullptr;       // first fragment unit of every 4-column tile (nft4 + 1)
  int *d_ew_crange = nullptr;     // column-range bounds of the force pass for 1..EW_MMA_MAXR ranges
  yg_occ ew_occ_fm;               // resident tensor-core force-pass blocks
  yg_occ ew_occ_s;                // resident warp-MMA S-pass blocks
  void *d_ew_te = nullptr;        // E0|E1 rows (float2), atoms padded to a multiple of 32
  void *d_ew_yf = nullptr;        // q E2 as FP16 (hi, lo) pairs per (atom, m)
  void *d_ew_ys = nullptr;        // q E2 per 16 atoms: FP16 B fragments, or the tcgen05 S-pass B operand
  void *d_ew_wb = nullptr;        // force weights as FP16 B fragments, per group
  size_t ew_bytes_te = 0, ew_bytes_yf = 0, ew_bytes_ys = 0, ew_bytes_wb = 0;
  // tcgen05 form of the force pass (yg_ewald_umma.cu): 64-column tiles
  int ew_umma = 0;                // 1 when the k-space layout suits it
  int ew_force_path = 0;          // requested: 0 automatic, 1 warp-level MMA
  int ew_sfac_path = 0;           // S pass requested: 0 automatic (warp-level MMA), 1 warp-level MMA, 2 tcgen05
  int ew_nut = 0;                 // 64-column tiles with work
  int ew_ubunits = 0;             // 16 KB B-operand units (tile x K-step) of one group's weights
  int *d_ew_uoff = nullptr;       // first unit of every 64-column tile (nut + 1)
  int *d_ew_upk = nullptr;        // the tiles' columns packed for the tcgen05 epilogue (-1: padding)
  float2 *d_ew_upf = nullptr;     // the tiles' columns' signed (g0, g1) as floats (0 for padding)
  int *d_ew_urange = nullptr;     // tile-range bounds for 1..EW_MMA_MAXR ranges
  void *d_ew_ya = nullptr;        // A operand (q E2 hi/lo) per 128-atom block and K-step
  void *d_ew_ub = nullptr;        // B operand (weights hi/lo) per unit, per group
  size_t ew_bytes_ya = 0, ew_bytes_ub = 0;
  int *d_ew_fpre = nullptr;       // prefix sums of the force column-tile costs (nftile + 1)
  double *d_ew_fpiece = nullptr;  // force sums of the split atom tiles [tile][part][NA][3]
  size_t ew_bytes_fpiece = 0;
  yg_occ ew_occ_f;                // resident force-pass blocks

  // valence
  int64_t ndelta = 0, nic = 0, nterm = 0;
  int2 *d_delta_ij = nullptr;
  double *d_delta = nullptr;      // ndelta*6: dx,dy,dz,gx,gy,gz
  int64_t *d_ic = nullptr;        // nic*9: kind, i0,s0,i1,s1,i2,s2,i3,s3
  double *d_icval = nullptr;      // nic*2: value, grad
  double *d_vpar = nullptr;       // nterm*6: par0..par5
  int4 *d_vkind = nullptr;        // nterm: term kind, ic0, ic1 (-1 unused), 0
  double *d_vE = nullptr;         // nterm

  // device-resident velocity Verlet (yg_md_*)
  double *d_vel = nullptr;        // natom*3
  double *d_invm = nullptr;       // natom
  double *d_md_ekpart = nullptr;
  double *d_md_ekin = nullptr;
  double *d_md_log = nullptr;     // (max_steps+1)*2: epot, ekin
  double *d_md_extra = nullptr;   // host-side energy added to epot (neutralizing term)
  // thermostat of the device step (0 none, 1 Berendsen, 2 Langevin, 3 CSVR,
  // 4 Nose-Hoover chain); state block: [0] conserved-energy correction,
  // [1] velocity factor, [2] kinetic energy before a stochastic update,
  // [3] chi-square sum, [8..15] chain positions, [16..23] chain velocities,
  // [24..31] chain masses
  int md_thermo = 0;
  double md_kT = 0.0, md_timecon = 0.0;
  int64_t md_ndof = 0;
  int md_nhc_len = 0;
  unsigned long long md_seed = 0;
  double *d_md_thermo = nullptr, *d_snap_thermo = nullptr;
  int *d_md_step = nullptr;
  double md_dt = 0.0;
  int md_mask = 0;
  int64_t md_max_steps = 0, md_steps_done = 0;
  int md_ready = 0;
  int md_graph_valid = 0;
  cudaGraphExec_t md_graph_exec = nullptr;
  cudaStream_t md_cap_stream = nullptr;  // capture stream of the step graph
  // control words of the device-driven step: [0] rebuild gate of this step,
  // [1] force a rebuild, [2] rebuilds so far, [4..5] pair count of the last
  // rebuild (u64), [6..7] largest squared displacement bits (u64)
  int *d_md_ctrl = nullptr;
  double *d_snap_pos = nullptr, *d_snap_vel = nullptr, *d_snap_total = nullptr;
  int *d_snap_step = nullptr;
  int64_t md_rebuilds = 0;        // rebuild count at the end of the last run
  double md_graph_skin = 0.0;

  // results per part: energy, vtens[9]; gpos natom*3
  double *d_part_ev = nullptr;    // YG_NPART*10
  double *d_part_gpos = nullptr;  // YG_NPART*natom*3
  double *d_total = nullptr;      // 10 + natom*3
  double *h_total = nullptr;      // pinned mirror
  cudaEvent_t rb_ev[YG_RB_CHUNKS] = {};  // chunks of the gradient readback
  cudaEvent_t build_ev = nullptr; // an enqueued build's status and count have arrived (h_status, h_u64[6])
  int build_pending = 0;          // a build was enqueued without waiting for its status
  double *h_total_dev = nullptr;  // device alias of h_total (page-locked, mapped), when the device has one
  int h_total_dev_state = 0;      // 0: not queried yet
  int ats_state = 0;              // device reads/writes pageable host memory: 1 yes, -1 no, 0 not queried yet
  double *d_red = nullptr;        // block partials for energy/virial reductions
  size_t red_cap = 0;
  int part_valid[YG_NPART] = {0, 0, 0, 0, 0, 0};
};

// ------------------------------------------------------------------ errors
void yg_set_error(const std::string &msg);
int yg_cuda_fail(cudaError_t err, const char *what);
#define YG_CUDA(call)                                   \
  do {                                                  \
    cudaError_t _e = (call);                            \
    if (_e != cudaSuccess) return yg_cuda_fail(_e, #call); \
  } while (0)
#define YG_LAUNCH_CHECK(ctx, what)                          \
  do {                                                      \
    (ctx)->launches++;                                      \
    cudaError_t _e = cudaGetLastError();                    \
    if (_e != cudaSuccess) return yg_cuda_fail(_e, what);   \
  } while (0)

// Device buffers are stream-ordered allocations on the context's stream from
// a per-device pool: creating and destroying contexts never synchronizes the
// device, so contexts on different streams run concurrently.
// Grows a device buffer to at least `bytes` (contents are not preserved).
int yg_ensure(yg_ctx *ctx, void **ptr, size_t *cap, size_t bytes);
// Makes the context's stream wait for a reciprocal sum still running on its
// auxiliary stream (no host synchronization).
int yg_ewald_join(yg_ctx *ctx);
int yg_alloc(yg_ctx *ctx, void **ptr, size_t bytes);
// Releases a buffer (stream-ordered) and clears the pointer.
void yg_free(yg_ctx *ctx, void **ptr);

// --------------------------------------------- exact FP64 (no contraction)
// These reproduce the operation order of the reference C code with every
// multiply and add rounded separately, as x86-64 SSE2 code does.
__device__ __forceinline__ double xmul(double a, double b) { return __dmul_rn(a, b); }
__device__ __forceinline__ double xadd(double a, double b) { return __dadd_rn(a, b); }
__device__ __forceinline__ double xsub(double a, double b) { return __dsub_rn(a, b); }

// Sequential fractional wrap of d; m receives the subtracted image
// (yaff/pes/cell.c:81-106).
__device__ __forceinline__ void exact_mic(double *d, const CellGeom &c, int *m) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double *g = c.gv + 3 * k;
    const double *r = c.rv + 3 * k;
    double x = ceil(xsub(xadd(xadd(xmul(g[0], d[0]), xmul(g[1], d[1])), xmul(g[2], d[2])), 0.5));
    d[0] = xsub(d[0], xmul(x, r[0]));
    d[1] = xsub(d[1], xmul(x, r[1]));
    d[2] = xsub(d[2], xmul(x, r[2]));
    m[k] = (int)x;
  }
}

// d += sum_k img[k] * rv[k], axis by axis (yaff/pes/cell.c:124-143).
__device__ __forceinline__ void exact_add_vec(double *d, const CellGeom &c, const int *img) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double *r = c.rv + 3 * k;
    double m = (double)img[k];
    d[0] = xadd(d[0], xmul(m, r[0]));
    d[1] = xadd(d[1], xmul(m, r[1]));
    d[2] = xadd(d[2], xmul(m, r[2]));
  }
}

// Image that brings d to the centre, all axes from the same d
// (yaff/pes/cell.c:109-121).
__device__ __forceinline__ void exact_to_center(const double *d, const CellGeom &c, int *ctr) {
#pragma unroll
  for (int k = 0; k < 3; k++) {
    const double *g = c.gv + 3 * k;
    ctr[k] = (int)(-ceil(xsub(xadd(xadd(xmul(g[0], d[0]), xmul(g[1], d[1])), xmul(g[2], d[2])), 0.5)));
  }
}

__device__ __forceinline__ double exact_norm2(const double *d) {
  return xadd(xadd(xmul(d[0], d[0]), xmul(d[1], d[1])), xmul(d[2], d[2]));
}

// Half space of images: first non-zero of (r2, r1, r0) is positive.
__device__ __forceinline__ bool img_positive(const int *r) {
  if (r[2] != 0) return r[2] > 0;
  if (r[1] != 0) return r[1] > 0;
  return r[0] > 0;
}

__device__ __forceinline__ bool img_zero(const int *r) {
  return r[0] == 0 && r[1] == 0 && r[2] == 0;
}

// ------------------------------------------------------- launchers (host)
int yg_launch_nlist_build(yg_ctx *ctx, double rc2, int *retry);
int yg_launch_nlist_build_async(yg_ctx *ctx, double rc2);
int yg_launch_nlist_build_wait(yg_ctx *ctx);
int yg_launch_nlist_build_gated(yg_ctx *ctx, const int *gate, unsigned long long *total);
int yg_launch_max_disp2_async(yg_ctx *ctx, unsigned long long *out);
int yg_launch_nlist_export(yg_ctx *ctx, yg_neigh_row *rows_host, int64_t cap, int64_t *n);
int yg_launch_prep_positions(yg_ctx *ctx);
int yg_launch_max_disp2(yg_ctx *ctx, double *out);
int yg_launch_pair(yg_ctx *ctx, int slot_mask, int want_grad);
int yg_launch_ewald_setup(yg_ctx *ctx);
int yg_launch_ewald_reci(yg_ctx *ctx, int want_grad);
int yg_launch_ewald_corr(yg_ctx *ctx, int want_grad);
int yg_launch_valence(yg_ctx *ctx, int want_grad);
int yg_launch_total(yg_ctx *ctx, int part_mask);
int yg_pack_pair_params(yg_ctx *ctx);
int yg_launch_reduce_ev(yg_ctx *ctx, const double *partials, int nblocks, int nval, double *out);
int yg_launch_check_wait_timeout(yg_ctx *ctx, int64_t polls);
// Raises a kernel's dynamic shared-memory limit once per (kernel, device).
int yg_smem_optin(const void *kernel, size_t need);
// tcgen05 force pass of the mixed reciprocal sum (yg_ewald_umma.cu)
size_t yg_umma_force_smem(int ne);
int yg_umma_kmax();
int yg_umma_cols();
int yg_launch_ya_umma(yg_ctx *ctx, const void *yf, int64_t a0, int64_t n, int nmf, int nks, int64_t nblk, void *ya);
int yg_launch_force_umma(yg_ctx *ctx, const void *te, const void *ya, int a0, int a1, int ne, int G0, int lep,
                         int nks, const int *urange, int nr, const void *ub, double inv1, double inv2, double *out,
                         int64_t rstride);
// tcgen05 S pass (yg_ewald_umma.cu)
size_t yg_umma_sfac_smem(int lep);
int yg_umma_sfac_atb();
int yg_launch_yb_umma(yg_ctx *ctx, const void *yf, int64_t lo, int64_t hi, int64_t base1, int64_t base2,
                      int64_t nblocks, int nmf, int nks, void *yb);
int yg_launch_sfac_umma(yg_ctx *ctx, const void *te, const void *yb, int n, int G0, int lep, int nks,
                        const void *cols, void *Spart, int ntile64, int sms);

// Grid-stride helper.
static inline int yg_blocks(int64_t n, int threads) {
  int64_t b = (n + threads - 1) / threads;
  if (b < 1) b = 1;
  if (b > (int64_t)1 << 30) b = (int64_t)1 << 30;
  return (int)b;
}
