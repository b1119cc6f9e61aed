/*
 * yaffgb.h -- C ABI of the GB300 force-evaluation library (libyaffgb.so).
 *
 * One yg_ctx holds the device-resident state of one periodic system: its
 * positions, cell, neighbour list, pair-potential parameters, exclusion
 * table, Ewald k-space tables and valence tables, and the per-part results of
 * the last evaluation.  Every entry point takes plain pointers and sizes,
 * returns a yg_status (never traps), and enqueues its work on the context's
 * stream.  Results are copied out with yg_get_part / yg_get_total.
 *
 * Conventions kept from the reference C core: atomic units; positions are
 * (natom, 3) row-major float64; cell vectors are rows of a 3x3 matrix and the
 * reciprocal vectors are rows of inv(rvecs)^T; the energy, gradient (gpos) and
 * virial (vtens) of a part are computed by the part and ADDED by the caller.
 *
 * Each declaration names the reference interface (file:line in the
 * reference project) that it replaces.
 */
#ifndef YAFFGB_H
#define YAFFGB_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct yg_ctx yg_ctx;

/* status codes */
#define YG_OK 0
#define YG_ERR_ARG 1            /* invalid argument (bad size, index, pointer) */
#define YG_ERR_CUDA 2           /* a CUDA runtime call failed */
#define YG_ERR_NAN 3            /* an energy, gradient or virial was NaN */
#define YG_ERR_UNSUPPORTED 4    /* feature outside the supported set */
#define YG_ERR_CAPACITY 5       /* a device buffer was too small (retried internally) */
#define YG_ERR_DENSITY 6        /* atom density too high for a neighbour-list build */
#define YG_ERR_STATE 7          /* call order violated (e.g. compute before build) */

/* precision of the pair and reciprocal-space terms */
#define YG_FP64 0          /* plain: FP64 throughout */
#define YG_MIXED 1         /* FP32 terms, FP64 accumulation */
#define YG_MIXED_KAHAN 2   /* FP32 terms, Kahan-compensated FP32 accumulation */

/* pair-potential kinds (yaff/pes/pair_pot.c:277, :321, :711; per-atom
 * parameters: LJ, MM3, EI, MM3CAP :373, Grimme :434) and the kinds whose
 * parameters are tables over pairs of atom types (ExpRep :473, QMDFFRep
 * :506, LJCross :540, DampDisp :596, Disp68BJDamp :651) */
#define YG_POT_LJ 0
#define YG_POT_MM3 1
#define YG_POT_EI 2
#define YG_POT_MM3CAP 3
#define YG_POT_GRIMME 4
#define YG_POT_EXPREP 5
#define YG_POT_QMDFFREP 6
#define YG_POT_LJCROSS 7
#define YG_POT_DAMPDISP 8
#define YG_POT_DISP68BJ 9

/* truncation kinds (yaff/pes/truncation.c:30, :59) */
#define YG_TR_NONE 0
#define YG_TR_HAMMER 1
#define YG_TR_SWITCH3 2

/* result slots for yg_get_part */
#define YG_PART_PAIR0 0    /* pair potentials 0..2 use slots 0..2 */
#define YG_PART_EWALD_RECI 3
#define YG_PART_EWALD_CORR 4
#define YG_PART_VALENCE 5
#define YG_NPART 6

/* One row of the exported neighbour list; same layout as the reference's
 * neigh_row_type (yaff/pes/nlist.h:30-35). */
typedef struct {
  int64_t a, b;
  double d, dx, dy, dz;
  int64_t r0, r1, r2;
} yg_neigh_row;

/* Human-readable text for a status code. */
const char *yg_status_string(int status);

/* Last error message recorded on this thread (for YG_ERR_CUDA / YG_ERR_ARG). */
const char *yg_last_error(void);

/* Creates a context for natom atoms on the current CUDA device; `stream` is a
 * cudaStream_t (NULL = legacy default stream).  No reference counterpart: the
 * reference keeps this state in Python objects (yaff/pes/ff.py:117-168,
 * yaff/pes/nlist.py:54-117). */
int yg_create(int64_t natom, int precision, void *stream, yg_ctx **out);
int yg_destroy(yg_ctx *ctx);
int yg_set_precision(yg_ctx *ctx, int precision);

/* Cell vectors and reciprocal vectors (rows, 3x3 host arrays) as computed by
 * the host cell object; replaces cell_update (yaff/pes/cell.c:37-79).  Only
 * nvec == 3 is supported by the device neighbour list. */
int yg_set_cell(yg_ctx *ctx, const double *rvecs, const double *gvecs, int nvec,
                double volume);

/* Copies positions (natom x 3 float64) into the context; `on_device` != 0
 * means `pos` is a device pointer.  The reference reads system.pos directly
 * (yaff/pes/ff.py:261-266). */
int yg_set_positions(yg_ctx *ctx, const double *pos, int on_device);

/* Per-atom charges (host, natom float64), used by EI and Ewald parts. */
int yg_set_charges(yg_ctx *ctx, const double *charges);

/* Exclusion / scaling table rows (a > b, scale, nbond), sorted by (a, b);
 * replaces the stab argument of pair_pot_compute (yaff/pes/pair_pot.c:84-87)
 * and compute_ewald_corr (yaff/pes/ewald.c:278-281). */
int yg_set_scalings(yg_ctx *ctx, const int64_t *a, const int64_t *b,
                    const double *scale, const int64_t *nbond, int64_t n);

/* Registers pair potential `slot` (0..2).  Arrays are host, natom long; NULL
 * when unused by the kind.  Replaces pair_data_lj_init / pair_data_mm3_init /
 * pair_data_ei_init and pair_pot_set_rcut / set_trunc_scheme
 * (yaff/pes/pair_pot.c:266-275, :308-319, :693-709, :48-58). */
int yg_set_pair_pot(yg_ctx *ctx, int slot, int kind, const double *sigma,
                    const double *epsilon, const int32_t *onlypauli,
                    const double *radii, double alpha, double dielectric,
                    double rcut, int tr_kind, double tr_par);

/* Registers a pair potential whose parameters are tables over pairs of atom
 * types (kinds YG_POT_EXPREP .. YG_POT_DISP68BJ).  ffatype_ids: natom type
 * indices in [0, nffatype); cross0/cross1/cross2: nffatype x nffatype
 * row-major tables (amp/b for ExpRep and QMDFFRep, eps/sig for LJCross, cn/b
 * for DampDisp, c6/c8/R for Disp68BJDamp; cross2 NULL except for the last);
 * power: the dispersion power of DampDisp; scales: {c6_scale, c8_scale,
 * bj_a, bj_b} of Disp68BJDamp, else NULL.  Replaces pair_data_exprep_init,
 * pair_data_qmdffrep_init, pair_data_ljcross_init, pair_data_dampdisp_init
 * and pair_data_disp68bjdamp_init (yaff/pes/pair_pot.c:458-471, :491-504,
 * :524-538, :560-574, :631-649). */
int yg_set_pair_table(yg_ctx *ctx, int slot, int kind, int64_t nffatype,
                      const int64_t *ffatype_ids, const double *cross0,
                      const double *cross1, const double *cross2, int64_t power,
                      const double *scales, double rcut, int tr_kind, double tr_par);
int yg_clear_pair_pots(yg_ctx *ctx);

/* Full neighbour-list rebuild for all pairs closer than rcut_total over the
 * half space of images |r_k| <= rmax[k], restricted by nlow/nhigh.  Writes the
 * number of half-list rows to *nneigh.  Replaces nlist_build_low plus the
 * grow-and-resume loop (yaff/pes/nlist.c:30-131, yaff/pes/nlist.py:163-186). */
int yg_nlist_build(yg_ctx *ctx, double rcut_total, const int64_t *rmax,
                   int64_t nlow, int64_t nhigh, int64_t *nneigh);

/* Per-atom neighbour-slot capacity of the next builds, rounded up to a
 * multiple of 32 (no reference counterpart; the reference grows its row
 * buffer the same way, yaff/pes/nlist.py:170-182).  The current list is
 * dropped: host computes need a new yg_nlist_build, and a device-resident MD
 * run rebuilds at its next step.  A build that needs more slots than this
 * regrows as usual (the host build reruns; the MD rolls its batch back to
 * the snapshot and reruns it). */
int yg_nlist_set_capacity(yg_ctx *ctx, int64_t slots);

/* Statistics of the last host-driven build (no reference counterpart):
 * candidates decided by the exact FP64 test (inside the FP32 guard band)
 * and the longest per-atom row of the device list (both directions). */
int yg_nlist_stats(yg_ctx *ctx, int64_t *nexact, int64_t *maxrow);

/* Layout of the reciprocal sum set up by yg_ewald_setup (no reference
 * counterpart): how the mixed forms run it -- 0 on the CUDA cores, 1 both
 * contractions as warp-level MMAs (needs G2 + 1 <= 32 and G0 + G1 + 2 <=
 * 160), 2 the force pass on tcgen05 with TMEM accumulators and the structure
 * factors as warp-level MMAs (also needs G0 + G1 + 2 <= 63) -- and the number
 * of k vectors in the half sphere. */
int yg_ewald_info(yg_ctx *ctx, int *tensor_path, int64_t *nk);

/* Failure-path self-check (no reference counterpart): runs the bounded
 * mbarrier wait used by the kernels that stage data with bulk copies on a
 * barrier nothing arrives at, giving up after `polls` polls (1 .. 2^24; the
 * kernels use 2^24, about a second).  *timed_out is set to 1 when the wait
 * gave up and recorded the timeout status, as it must; the context stays
 * usable. */
int yg_check_wait_timeout(yg_ctx *ctx, int64_t polls, int *timed_out);

/* Selects the kernel of the mixed-precision reciprocal force pass (no
 * reference counterpart): 0 automatic (tcgen05 where the layout allows), 1
 * the warp-level MMA form.  Both compute the same sums. */
int yg_ewald_force_path(yg_ctx *ctx, int path);

/* Selects the kernel of the mixed-precision structure-factor (S) pass (no
 * reference counterpart): 0 automatic (the warp-level MMA form, the faster
 * one on GB300), 1 the warp-level MMA form, 2 the tcgen05 form (TMEM
 * accumulators; where its staging does not fit, the warp-level form runs).
 * Both compute the same sums (FP16-split products, FP32 accumulation over
 * at most 32 atoms, chunk partials summed in a fixed order). */
int yg_ewald_sfac_path(yg_ctx *ctx, int path);

/* The reciprocal sum runs on an auxiliary stream of the context, forked at
 * yg_ewald_reci, so that it overlaps the neighbour build and the pair terms;
 * every call that reads its results or changes its inputs joins it back.
 * yg_ewald_wait makes the context's stream wait for it explicitly (no host
 * synchronization), e.g. to time it with events on the context's stream. */
int yg_ewald_wait(yg_ctx *ctx);

/* The same build enqueued without waiting for its outcome (nlist.c:30-180 as
 * yg_nlist_build): the pair terms can be enqueued behind it at once, so the
 * GPU does not idle while the host learns the row count.  yg_nlist_build_wait
 * returns its outcome: YG_OK with the reference's row count in *nneigh, or
 * YG_ERR_CAPACITY when a row overflowed its slots (the slot capacity is grown;
 * the rows and every pair result computed from them are invalid: build again,
 * e.g. with yg_nlist_build, and recompute), or YG_ERR_NAN for a position that
 * could not be binned.  yg_get_total, yg_get_part, yg_nlist_export,
 * yg_nlist_recompute and the MD entry points wait for it themselves and return
 * that error before they read anything the rows produced. */
int yg_nlist_build_async(yg_ctx *ctx, double rcut_total, const int64_t *rmax, int64_t nlow, int64_t nhigh);
int yg_nlist_build_wait(yg_ctx *ctx, int64_t *nneigh);

/* Skin path: keeps the pairs of the last rebuild and re-evaluates relative
 * vectors from the current positions.  Replaces nlist_recompute_low
 * (yaff/pes/nlist.c:183-232). */
int yg_nlist_recompute(yg_ctx *ctx);

/* Largest squared displacement since the last rebuild (for the skin test of
 * yaff/pes/nlist.py:207-218). */
int yg_nlist_max_disp2(yg_ctx *ctx, double *out);

/* Exports the current half list as reference rows, sorted by (a, b, r0, r1,
 * r2).  `rows` is host memory for `cap` rows; *n receives the row count (if
 * *n > cap nothing is written).  Replaces reading NeighborList.neighs
 * (yaff/pes/nlist.py:86-88). */
int yg_nlist_export(yg_ctx *ctx, yg_neigh_row *rows, int64_t cap, int64_t *n);

/* Evaluates the registered pair potentials (bit i of slot_mask = slot i) in
 * one pass over the neighbour list.  Replaces pair_pot_compute
 * (yaff/pes/pair_pot.c:84-176), one call per potential, with one fused
 * traversal; per-slot results go to result slots YG_PART_PAIR0 + slot. */
int yg_pair_compute(yg_ctx *ctx, int slot_mask, int want_grad);

/* Ewald reciprocal-space term over the half sphere |k| <= 2 pi gcut with
 * |g_k| <= gmax[k] and the nlow/nhigh split.  Replaces compute_ewald_reci
 * (yaff/pes/ewald.c:32-150). */
int yg_ewald_setup(yg_ctx *ctx, double alpha, double gcut, const int64_t *gmax,
                   double dielectric, int64_t nlow, int64_t nhigh);
int yg_ewald_reci(yg_ctx *ctx, int want_grad);

/* Ewald self term and excluded-pair double counting.  Replaces
 * compute_ewald_corr (yaff/pes/ewald.c:278-349). */
int yg_ewald_corr(yg_ctx *ctx, int want_grad);

/* Valence tables: relative vectors (i, j), internal coordinates (9 int64 per
 * row: kind 0..17, then delta row and sign for up to four deltas, as
 * iclist_row_type of yaff/pes/iclist.h:30-38) and energy terms (kind 0..15,
 * six parameters, two coordinate rows with -1 when unused, as vlist_row_type
 * of yaff/pes/vlist.h:30-37).  Replaces the DeltaList /
 * InternalCoordinateList / ValenceList tables (yaff/pes/dlist.py:62-118,
 * iclist.py:77-120, vlist.py:74-110). */
int yg_set_valence(yg_ctx *ctx, const int64_t *delta_ij, int64_t ndelta,
                   const int64_t *ic_rows, int64_t nic, const int64_t *vterm_kind,
                   const double *vterm_pars, const int64_t *vterm_ic, int64_t nterm);

/* Forward and back propagation of the valence chain.  Replaces dlist_forward
 * / iclist_forward / vlist_forward and vlist_back / iclist_back / dlist_back
 * (yaff/pes/dlist.c:29-69, iclist.c:314-320, :853-858, vlist.c:146-155,
 * :260-265). */
int yg_valence_compute(yg_ctx *ctx, int want_grad);

/* Reads back the result of one part: energy, gradient (natom x 3, may be
 * NULL) and virial (3x3, may be NULL) into host memory. */
int yg_get_part(yg_ctx *ctx, int part, double *energy, double *gpos, double *vtens);

/* Sums the parts in part_mask on the device and reads back the total energy,
 * gradient (may be NULL) and virial (may be NULL); per-part energies go to
 * part_energies[YG_NPART] when not NULL.  gpos is writable host memory of
 * 3 natom doubles: where the device reaches pageable host memory through
 * the host's page tables the device writes the gradient into it after
 * checking the result on the device, otherwise the host copies it from the
 * page-locked readback block.  A NaN or invalid result (YG_ERR_NAN,
 * YG_ERR_CUDA) leaves gpos and vtens untouched. */
int yg_get_total(yg_ctx *ctx, int part_mask, double *energy, double *gpos,
                 double *vtens, double *part_energies);

/* As yg_get_total, but the summed gradient and virial are ADDED to gpos and
 * vtens (yaff's ForcePart.compute convention, ff.py:117-168), by the device
 * or from the page-locked readback block as for yg_get_total, without an
 * intermediate copy. */
int yg_get_total_add(yg_ctx *ctx, int part_mask, double *energy, double *gpos,
                     double *vtens, double *part_energies);

/* Waits for all work queued on the context's stream. */
int yg_sync(yg_ctx *ctx);

/* Number of kernels this context has launched since creation. */
int64_t yg_launch_count(yg_ctx *ctx);

/* Device memory held by the context: bytes now and the high-water mark since
 * creation (no reference counterpart; the serving loop's admission check). */
int yg_mem_usage(yg_ctx *ctx, int64_t *bytes_now, int64_t *bytes_high);

/* The library's stream-ordered device pool on the current device (all
 * contexts allocate from it; creating and destroying contexts never
 * synchronizes the device): bytes in use, their high-water mark and bytes
 * reserved from the driver.  Any pointer may be NULL. */
int yg_pool_usage(int64_t *used_now, int64_t *used_high, int64_t *reserved);

/* Device-resident velocity Verlet of yaff/sampling/verlet.py:320-367 for the
 * serving loop: positions, velocities (host arrays here, natom x 3), masses
 * and the neighbour list stay in HBM.  part_mask selects the result slots
 * summed into the force (bit YG_PART_*); extra_energy is a constant added to
 * the logged potential energy (the host-side neutralizing term); the energy
 * log holds max_steps + 1 (epot, ekin) rows.  Requires a built list. */
int yg_md_setup(yg_ctx *ctx, const double *masses, const double *vel, double dt,
                int part_mask, double extra_energy, int64_t max_steps);

/* Runs nsteps steps without host synchronization inside a batch of up to
 * 128 steps: the skin test of yaff/pes/nlist.py:207-218 (rebuild when
 * 2 (rmax+1) max|r - r_build| >= skin; skin <= 0: every step) runs on the
 * device and gates the rebuild kernels.  With use_graph != 0 a whole step is
 * replayed from a CUDA graph captured on first use.  The host reads the
 * status words once per batch; a batch in which a rebuilt neighbour row
 * overflowed its slot is rolled back and run again with larger slots.
 * *nrebuild receives the number of rebuilds. */
int yg_md_run(yg_ctx *ctx, int64_t nsteps, int use_graph, double skin, int64_t *nrebuild);

/* Copies positions, velocities (natom x 3) and the energy log
 * ((*nlog) x 2) to host memory; any pointer may be NULL. */
int yg_md_get(yg_ctx *ctx, double *pos, double *vel, double *log, int64_t *nlog);

/* Thermostat of the device step, applied where the reference calls its
 * Verlet hooks: kind 0 none, 1 Berendsen (before the first half kick), 2
 * Langevin (before and after), 3 CSVR (before), 4 Nose-Hoover chain (before
 * and after).  kT = k_B T0, timecon the time constant, ndof the degrees of
 * freedom; a chain of 1..8 beads takes its positions, velocities and masses;
 * the Langevin and CSVR noise comes from a counter-based generator keyed by
 * `seed` and the step number.  Replaces BerendsenThermostat,
 * LangevinThermostat, CSVRThermostat and NHCThermostat with NHChain
 * (yaff/sampling/nvt.py:110-270, :346-500) for yg_md_run.  Call after
 * yg_md_setup (which resets it to none). */
int yg_md_thermostat(yg_ctx *ctx, int kind, double kT, double timecon, int64_t ndof, int chain_length,
                     const double *chain_pos, const double *chain_vel, const double *chain_masses,
                     unsigned long long seed);

/* The thermostat's conserved-energy correction (the sum the reference keeps
 * in VerletHook.econs_correction) and the chain positions / velocities; any
 * pointer may be NULL. */
int yg_md_thermo_get(yg_ctx *ctx, double *econs_correction, double *chain_pos, double *chain_vel);

/* Ewald correction for callers that cannot let the library allocate device
 * memory (an engine that owns all device memory through its own pool, or a
 * step loop that must not block on an allocation).  No counterpart in the
 * reference.  Computes what yg_ewald_corr computes -- the self term over
 * [nlow, nhigh) and the excluded-pair correction of the scaling rows
 * (stab_a > stab_b, stab_scale) -- from caller-owned DEVICE buffers: pos
 * (natom x 3), charges (natom), stab_* (nstab), and writes the energy
 * (1 double), the gradient gpos (natom x 3, overwritten; may be NULL) and
 * the virial vtens (9 doubles), all device memory, on `stream`.  rvecs and
 * gvecs are host 3x3 arrays; nhigh = -1 means natom, as in the reference.
 * Its only scratch is a fixed 256 KB device array inside the library, so
 * nstab is limited to YG_NOALLOC_MAX_ROWS (larger tables return
 * YG_ERR_CAPACITY).  The scaling rows are checked on the device: a row whose
 * indices are not 0 <= stab_b < stab_a < natom is skipped without touching
 * memory through it, and the call then stores a NaN energy.  The first call
 * on a device looks up that array's device address; make it before capturing
 * the stream in a graph.  All calls share the array: calls that overlap on
 * the GPU race and must be serialized by the caller. */
#define YG_NOALLOC_MAX_ROWS (1 << 20)
int yg_ewald_corr_noalloc(const double *pos, const double *charges, int64_t natom,
                          const int64_t *stab_a, const int64_t *stab_b,
                          const double *stab_scale, int64_t nstab,
                          const double *rvecs, const double *gvecs, double volume,
                          double alpha, double dielectric, int64_t nlow, int64_t nhigh,
                          double *energy, double *gpos, double *vtens, void *stream);

/* ------------------------------------------- many small systems (fleet) */

/* A fleet steps many independent small periodic systems -- the serving
 * workload: LJ + point-charge EI + Ewald, velocity Verlet -- with one launch
 * per phase of the MD step for all systems in flight (eight launches per
 * step, replayed from a CUDA graph), instead of one context and one launch
 * sequence per system.  Capacities are fixed at creation (atoms, systems,
 * k vectors, neighbour slots per atom, steps per system); systems are added
 * and removed between steps.  Each system follows the reference's physics
 * (pair_pot.c:277-301, :724-735; ewald.c:32-150, :289-292; ff.py:633-669;
 * verlet.py:339-367; the skin rule of nlist.py:207-218) with FP32 pair terms,
 * phases and structure factors and FP64 positions, velocities and energies;
 * its trajectory does not depend on the other systems in flight.  No
 * reference counterpart (the reference steps one system per process). */
typedef struct yg_fleet yg_fleet;
int yg_fleet_create(int64_t max_atoms, int max_systems, int64_t max_k, int max_neighbors, int max_steps,
                    void *stream, yg_fleet **out);
int yg_fleet_destroy(yg_fleet *fleet);
/* Adds a system of natom atoms (host arrays: pos and vel natom x 3, masses,
 * charges, LJ sigma and epsilon per atom (Lorentz-Berthelot mixing), the 3x3
 * cell rvecs) with cutoff rcut, Verlet skin, Ewald alpha and gcut, time step
 * dt and nsteps steps to run; *slot receives its slot.  YG_ERR_CAPACITY
 * when a slot, the atom range or the k range does not fit; YG_ERR_ARG when
 * rcut + skin needs more than two periodic images per cell axis, or when the
 * reciprocal-lattice extents need more than 64 phase-table entries per atom
 * ((G0 + 1) + (G1 + 1) + (G2 + 1), G_k = ceil(gcut |r_k| - 1/2)). */
int yg_fleet_add(yg_fleet *fleet, int64_t natom, const double *pos, const double *vel, const double *masses,
                 const double *charges, const double *sigma, const double *epsilon, const double *rvecs,
                 double rcut, double skin, double alpha, double gcut, double dt, int64_t nsteps, int *slot);
/* Frees a slot and its ranges (after yg_fleet_get). */
int yg_fleet_remove(yg_fleet *fleet, int slot);
/* Advances every stepping system by up to nsteps steps (each stops at its
 * own step count); enqueued on the fleet's stream. */
int yg_fleet_step(yg_fleet *fleet, int64_t nsteps);
/* Per slot (max_systems entries each, either may be NULL): state (0 empty,
 * 1 stepping, 2 done, 3 failed: a neighbour row overflowed) and completed
 * steps.  Waits for the fleet's stream. */
int yg_fleet_poll(yg_fleet *fleet, int *state, int *steps);
/* Positions, velocities (natom x 3) and the energy log ((steps + 1) x
 * (epot, ekin), step 0 first) of a slot; any pointer may be NULL.  Returns
 * YG_ERR_CAPACITY for a failed system. */
int yg_fleet_get(yg_fleet *fleet, int slot, double *pos, double *vel, double *log, int64_t *nlog);
/* Atom and k-vector capacity in use and the number of occupied slots. */
int yg_fleet_usage(yg_fleet *fleet, int64_t *atoms_used, int *systems_used, int64_t *k_used);
/* Kernel launches issued by the fleet so far (eight per step). */
int64_t yg_fleet_launch_count(yg_fleet *fleet);

/* ------------------------------------------------ MC trial energies ---- */

/* compute_ewald_prefactors (yaff/pes/ewald.c:441-471): fac1 exp(-k^2/4a^2)/k^2
 * for every k of the half sphere |k| <= 2 pi gcut, in the reference's dense
 * layout (2 gmax0+1) x (2 gmax1+1) x (gmax2+1) with the element of each k one
 * position after its loop index (ewald.c:457); prefactors must hold that
 * many doubles and is overwritten where k is inside the cutoff (the
 * reference writes one element past the array when the last loop index is
 * inside the cutoff; that element is dropped here).  Host FP64 set-up. */
int yg_ewald_prefactors(const double *gvecs, double volume, double alpha,
                        const int64_t *gmax, double gcut, double *prefactors);

/* compute_ewald_structurefactors (ewald.c:473-506): q cos(k.r) and q sin(k.r)
 * summed over the atoms, ADDED to cosfacs / sinfacs (host arrays, same dense
 * layout).  Evaluated on the GPU in FP64 on `stream`. */
int yg_ewald_structurefactors(const double *pos, int64_t natom, const double *charges,
                              const double *rvecs, const double *gvecs, double volume,
                              const int64_t *gmax, double gcut, double *cosfacs,
                              double *sinfacs, void *stream);

/* compute_ewald_deltae (ewald.c:508-522): 2 sum pref (cos dcos + sin dsin)
 * over nk elements of host arrays, on the GPU. */
int yg_ewald_deltae(const double *prefactors, const double *deltacosfacs,
                    const double *cosfacs, const double *deltasinfacs,
                    const double *sinfacs, int64_t nk, double *out);

/* Batched trial energies of rigid-guest moves (the trial path of
 * yaff/sampling/mctrials.py:69-126 with reci_ei = 'ewald_interaction',
 * mc.py:596-597).  A context holds a rigid framework (nframe atoms with
 * charges and LJ sigma/epsilon), the guest template (guest_natom <= 4
 * atoms) and nchain chains of up to max_guests guests each, with each
 * chain's structure factors resident in HBM.  rmax: real-space image range
 * (ceil(rcut/spacing - 0.5)); close_contact: the reference's close-contact
 * distance (a side of a trial within it counts 1e10; negative: off).
 * precision: YG_FP64 or YG_MIXED (FP32 pair terms and sincos on FP64
 * relative vectors and reduced phases, FP64 sums). */
typedef struct yg_mc yg_mc;
int yg_mc_create(const double *rvecs, const double *gvecs, double volume, const int64_t *rmax,
                 double rcut, double alpha, double gcut, const int64_t *gmax, double dielectric,
                 double close_contact, int64_t nframe, const double *frame_pos,
                 const double *frame_charges, const double *frame_sigma,
                 const double *frame_epsilon, int64_t guest_natom, const double *guest_charges,
                 const double *guest_sigma, const double *guest_epsilon, int64_t nchain,
                 int64_t max_guests, int precision, void *stream, yg_mc **out);
int yg_mc_destroy(yg_mc *mc);
int yg_mc_set_precision(yg_mc *mc, int precision);
/* Sets a chain's guests (nguest x guest_natom x 3 host positions) and
 * recomputes its structure factors (framework + guests). */
int yg_mc_set_chain(yg_mc *mc, int64_t chain, int64_t nguest, const double *guest_pos);
/* Reads a chain back: guest count, positions and structure factors in the
 * reference's dense layout (any pointer may be NULL). */
int yg_mc_get_chain(yg_mc *mc, int64_t chain, int64_t *nguest, double *guest_pos,
                    double *cosfacs, double *sinfacs);
/* The prefactor array of the context (dense layout; *nk_dense elements). */
int yg_mc_prefactors(yg_mc *mc, double *prefactors, int64_t *nk_dense);
/* Energy differences of ntrial trials (host arrays): kind 0 inserts a guest
 * at newpos, 1 deletes guest `guest`, 2 translates guest `guest` to newpos
 * (newpos: ntrial x guest_natom x 3, rows of deletions ignored).  Each is the
 * reference's U(after) - U(before) against the chain's current state: the
 * guest's LJ + real-space EI with the framework and the other guests and
 * its reciprocal interaction through the structure factors. */
int yg_mc_trials(yg_mc *mc, int64_t ntrial, const int32_t *chain, const int32_t *kind,
                 const int32_t *guest, const double *newpos, double *energy);
/* Accepts trials of the last batch (at most one per chain): positions and
 * structure factors are updated on the device as the reference's accept()
 * does (mctrials.py:177-190); a deletion moves the chain's last guest into
 * the freed slot. */
int yg_mc_apply(yg_mc *mc, int64_t napply, const int32_t *trial_index);
int64_t yg_mc_launch_count(yg_mc *mc);

#ifdef __cplusplus
}
#endif

#endif
