"""Benchmark: force evaluations per second on the 50,000-atom triclinic
MM3 + EI + Ewald workload (rcut 12 A, skin 1 A, alpha_scale 3.5,
gcut_scale 1.1), one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gb300|reference]
                    [--precision mixed|fp64|mixed_kahan] [--natom 50000]

A step is one ForceField.compute(gpos, vtens) of the whole system with a full
neighbour-list rebuild (every step moves the atoms, so nothing is reused).
`value`: device-resident inputs (positions already in HBM), CUDA-event
timed per step with an L2 flush between steps outside the timed events.
`e2e`: the same evaluation through the public Python API with host numpy
positions in and gradient/virial/energy out (H2D + D2H inside the timing).
Under torchrun every rank runs an independent replica (the path does not
shard); rank 0 prints the JSON line.
"""
import argparse
import ctypes
import json
import os
import subprocess
import sys
import threading
import time

import numpy as np

REPO = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, REPO)

from yaff_gb300 import replicas  # noqa: E402


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument('--gpus', type=int, default=1)
    ap.add_argument('--steps', type=int, default=20)
    ap.add_argument('--warmup', type=int, default=3)
    ap.add_argument('--impl', default='gb300', choices=['gb300', 'reference'])
    ap.add_argument('--precision', default='mixed', choices=['mixed', 'fp64', 'mixed_kahan'])
    ap.add_argument('--natom', type=int, default=50000)
    ap.add_argument('--fp64-steps', type=int, default=3)
    ap.add_argument('--no-cpu-baseline', action='store_true')
    ap.add_argument('--no-sweep', action='store_true', help='skip the precision sweep against the reference fixture')
    ap.add_argument('--serving-requests', type=int, default=4096,
                    help='requests of the serving workload run after the main measurement (0: skip)')
    ap.add_argument('--serving-rate', type=float, default=200.0, help='Poisson arrival rate, requests/s')
    ap.add_argument('--serving-slots', type=int, default=16)
    ap.add_argument('--serving-fleet-only', action='store_true',
                    help='serving: the fleet engine only (no per-context engine, no sequential FP64 baseline)')
    ap.add_argument('--mc-rounds', type=int, default=10, help='MC trial-energy batches per precision (0: skip)')
    ap.add_argument('--nve-steps', type=int, default=1000, help='steps of the 24,000-atom water NVE run (0: skip)')
    ap.add_argument('--sfac-path', type=int, default=0, choices=[0, 1, 2],
                    help='structure-factor pass of the main workload: 0 automatic (warp-level MMA), '
                         '1 warp-level MMA, 2 tcgen05')
    return ap.parse_args()


class ClockSampler(object):
    """nvidia-smi clock / throttle sampling during the timed region."""

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None
        self.thread = None

    def start(self):
        q = ('index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,'
             'clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,'
             'clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap')
        try:
            self.proc = subprocess.Popen(['nvidia-smi', '-i', str(self.index), '--query-gpu=' + q,
                                          '--format=csv,noheader,nounits', '-lms', '200'],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except OSError:
            self.proc = None
            return

        def reader():
            for line in self.proc.stdout:
                self.rows.append([x.strip() for x in line.split(',')])
        self.thread = threading.Thread(target=reader, daemon=True)
        self.thread.start()

    def stop(self):
        if self.proc is None:
            return {'sm_mhz': None, 'sm_max_mhz': None, 'reasons': ['nvidia-smi unavailable']}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm = [float(r[1]) for r in self.rows if len(r) >= 9 and r[1].replace('.', '').isdigit()]
        smax = [float(r[2]) for r in self.rows if len(r) >= 9 and r[2].replace('.', '').isdigit()]
        reasons = set()
        names = ['hw_slowdown', 'hw_thermal_slowdown', 'sw_thermal_slowdown', 'sw_power_cap']
        for r in self.rows:
            if len(r) < 9:
                continue
            for k, nm in enumerate(names):
                if r[5 + k].lower().startswith('active'):
                    reasons.add(nm)
        return {'sm_mhz': float(np.median(sm)) if sm else None, 'sm_max_mhz': max(smax) if smax else None,
                'reasons': sorted(reasons), 'samples': len(sm)}


def dist_setup():
    from yaff_gb300.replicas import dist_env
    return dist_env()


def peaks():
    path = os.path.join(REPO, 'MEASURED_PEAKS.json')
    if os.path.exists(path):
        with open(path) as fh:
            d = json.load(fh)
        return d, 'measured'
    return {'hbm_gbs': 6800.0, 'bf16_tflops': 1900.0}, 'fallback'


_probe = None


def probe_lib():
    """The bench-only throughput probes (yaff_gb300/csrc/bench/yg_probe.cu,
    built by yaff_gb300.build.build_probe; not part of libyaffgb.so):
    double yg_probe_peak(int kind, cudaStream_t)."""
    global _probe
    if _probe is None:
        import ctypes
        from yaff_gb300 import build
        _probe = ctypes.CDLL(build.build_probe())
        _probe.yg_probe_peak.restype = ctypes.c_double
        _probe.yg_probe_peak.argtypes = [ctypes.c_int, ctypes.c_void_p]
    return _probe


def fp32_fma_peak(torch):
    """FP32 CUDA-core peak (TFLOP/s, FMA = 2 flops) measured with FMA-chain
    kernels of the library, scalar, packed f32x2 and the two interleaved:
    (peak, {kind: TFLOP/s}), peak = the largest.  The measured-peaks file
    holds only HBM and bf16 tensor figures, and the pair and Ewald kernels
    use neither."""
    import ctypes
    lib = probe_lib()
    st = ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)
    both = {'scalar': float(lib.yg_probe_peak(0, st)), 'f32x2': float(lib.yg_probe_peak(2, st)),
            'f32x2+scalar': float(lib.yg_probe_peak(3, st))}
    v = max(both.values())
    return (v if v > 0 else None), both


def warp_mma_peak(torch):
    """Warp-level FP16 MMA (m16n8k16, FP32 accumulate) throughput in
    TFLOP/s, measured with an MMA-chain kernel of the library: the ceiling of
    the instruction the tensor-core Ewald kernels use."""
    import ctypes
    lib = probe_lib()
    v = float(lib.yg_probe_peak(5, ctypes.c_void_p(torch.cuda.current_stream().cuda_stream)))
    return v if v > 0 else None


def run_gb300(args, world, rank, local):
    import torch
    torch.cuda.set_device(local)
    import yaff_gb300
    from yaff_gb300 import configs, _lib
    spec = configs.triclinic_mm3_ei(natom=args.natom) if args.natom != 50000 else configs.triclinic_50000()
    natom = len(spec['pos'])
    rng = np.random.default_rng(7 + rank)
    ff = yaff_gb300.build_forcefield(spec, precision=args.precision)
    dev = yaff_gb300.device_of(ff.system)
    _lib.check(dev.lib.yg_ewald_sfac_path(dev.ctx, args.sfac_path), 'yg_ewald_sfac_path')
    stream = torch.cuda.current_stream()
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device='cuda')
    pos0 = spec['pos'].copy()
    gpos = np.zeros((natom, 3))
    vtens = np.zeros((3, 3))

    def positions(step):
        # a fresh small displacement per step: the list is rebuilt every step
        return pos0 + rng.uniform(-0.05, 0.05, pos0.shape)

    # --- device-resident value: positions staged in HBM before the timing ---
    dpos = [torch.tensor(positions(s), dtype=torch.float64, device='cuda')
            for s in range(args.warmup + args.steps)]

    def device_step(s, rebuild=True, defer=True):
        # the order of ForceField.compute's fused path: positions, the
        # reciprocal sum (forked onto its own stream), list, pairs, the rest
        dev.upload_positions_device(dpos[s].data_ptr())
        mask = 0
        for p in ff.parts:
            if isinstance(p, yaff_gb300.ForcePartEwaldReciprocal):
                p._launch(True)
                mask |= 1 << p.device_slot
        if rebuild:
            ff.nlist.rebuild_next = True   # full neighbour-list rebuild every step
        ff.nlist.update(upload=False, defer=defer)   # enqueued; the readback reports an overflow
        pmask = 0
        for p in ff.parts:
            if isinstance(p, yaff_gb300.ForcePartPair):
                pmask |= 1 << p._register()
        _lib.check(dev.lib.yg_pair_compute(dev.ctx, pmask, 1), 'pair')
        mask |= pmask
        for p in ff.parts:
            if p.device_slot is not None and not isinstance(p, (yaff_gb300.ForcePartPair,
                                                                 yaff_gb300.ForcePartEwaldReciprocal)):
                p._launch(True)
                mask |= 1 << p.device_slot
        return mask

    def step_total(s, rebuild=True, g=None, v=None):
        # one evaluation and its readback; a deferred rebuild that overflowed a
        # row (its capacity has grown) is redone with a waiting rebuild
        mask = device_step(s, rebuild)
        try:
            dev.get_total(mask, g, v)
        except _lib.YaffGBError as exc:
            if exc.status != _lib.YG_ERR_CAPACITY:
                raise
            ff.nlist._pending = False
            mask = device_step(s, True, defer=False)
            dev.get_total(mask, g, v)
        return mask

    for s in range(args.warmup):
        mask = step_total(s, True, gpos, vtens)
    torch.cuda.synchronize()
    if world > 1:
        torch.distributed.barrier()
    launches0 = dev.launch_count()
    nrebuild0 = ff.nlist.nrebuild
    clocks = ClockSampler(local)
    clocks.start()
    times = []
    ewald_times = []
    for s in range(args.warmup, args.warmup + args.steps):
        flush.fill_(float(s))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        mask = step_total(s)
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1) * 1e-3)
    nrebuild_timed = ff.nlist.nrebuild
    launches = dev.launch_count() - launches0
    # skin path (the neighbour list of the last rebuild is reused, as yaff
    # does while displacements stay inside the skin)
    skin_times = []
    for s in range(args.warmup, args.warmup + args.steps):
        flush.fill_(float(s))
        e0 = torch.cuda.Event(enable_timing=True)
        e1 = torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        mask = step_total(s, rebuild=False)
        e1.record(stream)
        torch.cuda.synchronize()
        skin_times.append(e0.elapsed_time(e1) * 1e-3)
    # per-phase timing of a full evaluation (L2 flushed first), one phase
    # after the other (in the timed steps the reciprocal sum overlaps the
    # other two on its own stream): neighbour build, pair terms,
    # reciprocal-space sum -- the three dominant parts
    reci = [p for p in ff.parts if isinstance(p, yaff_gb300.ForcePartEwaldReciprocal)][0]
    phase_times = {'neighbour_build': [], 'pair': [], 'ewald_reciprocal': []}
    for s in range(args.warmup, args.warmup + 5):
        flush.fill_(float(s))
        ev = [torch.cuda.Event(enable_timing=True) for _ in range(4)]
        dev.upload_positions_device(dpos[s % len(dpos)].data_ptr())
        ff.nlist.rebuild_next = True
        ev[0].record(stream)
        ff.nlist.update(upload=False)
        ev[1].record(stream)
        pmask = 0
        for p in ff.parts:
            if isinstance(p, yaff_gb300.ForcePartPair):
                pmask |= 1 << p._register()
        _lib.check(dev.lib.yg_pair_compute(dev.ctx, pmask, 1), 'pair')
        ev[2].record(stream)
        reci._launch(True)
        _lib.check(dev.lib.yg_ewald_wait(dev.ctx), 'yg_ewald_wait')
        ev[3].record(stream)
        torch.cuda.synchronize()
        for k, name in enumerate(('neighbour_build', 'pair', 'ewald_reciprocal')):
            phase_times[name].append(ev[k].elapsed_time(ev[k + 1]) * 1e-3)
    ewald_times = phase_times['ewald_reciprocal']
    clk = clocks.stop()
    t_step = float(np.mean(times))
    # independent replicas: the slowest rank's time (no collective in the steps)
    total = replicas.max_over_ranks(sum(times))
    value = world * args.steps / total

    # --- e2e through the public API: host numpy positions in, gradient out ---
    e2e_times = []
    for s in range(args.warmup + args.steps):
        p = positions(s)
        flush.fill_(float(s))
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        ff.update_pos(p)
        ff.nlist.rebuild_next = True   # same work as the device-resident steps
        gpos[:] = 0.0
        vtens[:] = 0.0
        ff.compute(gpos, vtens)
        t1 = time.perf_counter()
        if s >= args.warmup:
            e2e_times.append(t1 - t0)
    e2e = world * args.steps / float(sum(e2e_times))

    # plain FP64 form on the same workload (few steps: GB300 FP64 is slow)
    fp64 = None
    if args.precision != 'fp64' and args.fp64_steps > 0:
        dev.set_precision('fp64')
        for s in range(1):
            mask = step_total(s)
        torch.cuda.synchronize()
        tt = []
        for s in range(args.fp64_steps):
            flush.fill_(float(s))
            e0 = torch.cuda.Event(enable_timing=True)
            e1 = torch.cuda.Event(enable_timing=True)
            e0.record(stream)
            mask = step_total(s)
            e1.record(stream)
            torch.cuda.synchronize()
            tt.append(e0.elapsed_time(e1) * 1e-3)
        fp64 = 1.0 / float(np.mean(tt))
        dev.set_precision(args.precision)

    # precision sweep: every form's speed on this workload and its error
    # against the reference's own FP64 evaluation of the same positions
    sweep = None if args.no_sweep else precision_sweep(ff, dev, spec, args, step_total, stream, flush, fp64,
                                                         1.0 / t_step)

    pk, pk_src = peaks()
    nk = ff_nk(ff)
    fp32_peak, fp32_probe = fp32_fma_peak(torch)
    mma_probe = warp_mma_peak(torch)
    nat_scale = natom / 50000.0
    rooflines = {}
    # (c) reciprocal-space sum: 18 flops per atom*k of the reference's direct sum
    t_reci = float(np.mean(phase_times['ewald_reciprocal']))
    flops = 18.0 * natom * nk
    tcode = ctypes.c_int()
    _lib.check(dev.lib.yg_ewald_info(dev.ctx, ctypes.byref(tcode), None), 'yg_ewald_info')
    if tcode.value == 2:
        rooflines['ewald_reciprocal'] = {
            'bound': 'tensor', 'achieved': flops / t_reci / 1e12, 'unit': 'TFLOP/s', 'peak': pk['bf16_tflops'],
            'peak_source': pk_src + ' dense bf16 (burst)', 'frac': flops / t_reci / 1e12 / pk['bf16_tflops'],
            'kernel': 'k_tables_mma + ' + ('k_yb_umma + k_sfac_umma (S pass, tcgen05)' if args.sfac_path == 2
                                            else 'k_ys_mma + k_sfac_mma (S pass, warp MMA)') +
                      ' + k_ya_umma + k_ewald_force_umma (force pass, tcgen05 with TMEM accumulators) + '
                      'combine/gpos; FP16 hi/lo split, FP32 accumulate',
            'ms': t_reci * 1e3, 'units': {'atom_k': natom * nk, 'flops_per_atom_k': 18},
            'warp_mma_f16_peak_tflops': mma_probe,
            'traffic': 82.7e6 * nat_scale,
            'traffic_source': 'ncu dram read+write of k_sfac_mma (33.7 MB) + k_ya_umma (12.8 MB) + '
                              'k_ewald_force_umma (36.2 MB) at 50,000 atoms' +
                              ('' if natom == 50000 else ', scaled by atoms')}
    elif tcode.value == 1:
        rooflines['ewald_reciprocal'] = {
            'bound': 'tensor', 'achieved': flops / t_reci / 1e12, 'unit': 'TFLOP/s', 'peak': pk['bf16_tflops'],
            'peak_source': pk_src + ' dense bf16 (burst)', 'frac': flops / t_reci / 1e12 / pk['bf16_tflops'],
            'kernel': 'k_sfac_mma + k_ewald_force_mma (warp MMA, FP16 hi/lo split, FP32 accumulate) + tables/reduce',
            'ms': t_reci * 1e3, 'units': {'atom_k': natom * nk, 'flops_per_atom_k': 18},
            'tensor_flops_executed_per_atom_k': 72,
            'tensor_tflops_executed': 72.0 * natom * nk / t_reci / 1e12,
            'warp_mma_f16_peak_tflops': mma_probe,
            'frac_of_warp_mma_peak': (72.0 * natom * nk / t_reci / 1e12 / mma_probe) if mma_probe else None,
            'traffic': 76.3e6 * nat_scale,
            'traffic_source': 'ncu dram read+write of k_sfac_mma (40.3 MB) + k_ewald_force_mma (36.0 MB) at 50,000 '
                              'atoms' + ('' if natom == 50000 else ', scaled by atoms')}
    else:
        rooflines['ewald_reciprocal'] = {
            'bound': 'fp32' if args.precision != 'fp64' else 'fp64', 'achieved': flops / t_reci / 1e12,
            'unit': 'TFLOP/s', 'peak': fp32_peak, 'peak_source': 'FP32 FMA-chain kernels in bench.py',
            'frac': flops / t_reci / 1e12 / fp32_peak if fp32_peak else None,
            'kernel': 'k_sfac + k_ewald_force (CUDA cores)', 'ms': t_reci * 1e3,
            'units': {'atom_k': natom * nk, 'flops_per_atom_k': 18}, 'traffic': None}
    # (a) neighbour build: 24 B per atom (positions) + 8 B per half-list row
    t_build = float(np.mean(phase_times['neighbour_build']))
    nrow = int(ff.nlist.nneigh)
    bbytes = 24.0 * natom + 8.0 * nrow
    rooflines['neighbour_build'] = {
        'bound': 'hbm', 'achieved': bbytes / t_build / 1e9, 'unit': 'GB/s', 'peak': pk['hbm_gbs'],
        'peak_source': pk_src, 'frac': bbytes / t_build / 1e9 / pk['hbm_gbs'],
        'kernel': 'k_bin + k_scan_cells + k_scatter + k_sort_cells + k_origins + k_prep + k_build (full rows, '
                  'entries within the pair cutoff at the front and the skin shell at the back, exact FP64 '
                  'decisions in the FP32 guard band)',
        'ms': t_build * 1e3, 'units': {'rows': nrow, 'bytes': bbytes},
        'traffic': 312.8e6 * nat_scale,
        'traffic_source': 'ncu dram read+write of k_build (the candidate sweep) at 50,000 atoms (6.0 MB read, 306.8 '
                          'MB written): it writes both directions of every pair' +
                          ('' if natom == 50000 else ', scaled by atoms')}
    # (b) pair terms: 75 flops (+3 transcendentals) per half-list pair within rcut; the pairs within rcut
    # are estimated from the list by the (rcut / (rcut + skin))^3 volume ratio
    t_pair = float(np.mean(phase_times['pair']))
    rcut, skin = float(spec['rcut']), float(spec['skin'])
    npair = nrow * (rcut / (rcut + skin)) ** 3
    rooflines['pair'] = {
        'bound': 'fp32', 'achieved': 75.0 * npair / t_pair / 1e12, 'unit': 'TFLOP/s', 'peak': fp32_peak,
        'peak_source': 'FP32 FMA-chain kernels in bench.py (measured-peaks file has no FP32 figure)',
        'frac': (75.0 * npair / t_pair / 1e12 / fp32_peak) if fp32_peak else None,
        'kernel': 'k_pair<MM3, EI> (one warp per atom over its full row; each pair is evaluated from both ends; '
                  'on a fresh list the skin shell at the back of the row is not read)',
        'ms': t_pair * 1e3, 'units': {'pairs_within_rcut': npair, 'flops_per_pair': 75, 'transcendentals_per_pair': 3},
        'traffic': 300.7e6 * nat_scale,
        'traffic_source': 'ncu dram read+write of k_pair at 50,000 atoms (295.9 MB read, 4.8 MB written; the '
                          'skin shell is not read on a fresh list)' + ('' if natom == 50000 else ', scaled by atoms')}
    dom = max(rooflines, key=lambda k: rooflines[k]['ms'])
    roof = dict(rooflines[dom])
    roof['name'] = dom
    roof['fp32_peak_probe_tflops'] = fp32_probe
    lat = np.array(times) * 1e3
    out = {
        'metric': 'force evals/s', 'value': value, 'unit': 'evals/s', 'n_gpus': world, 'steps': args.steps,
        'warmup': args.warmup, 'ms_per_step': t_step * 1e3, 'higher_is_better': True, 'scaling': 'weak',
        'vs_baseline': None, 'dtype': {'mixed': 'fp32-terms/fp64-accum', 'fp64': 'f64',
                                        'mixed_kahan': 'fp32-kahan'}[args.precision],
        'data': 'synthetic (seeded random sequential insertion)',
        'config': workload_config(natom),
        'details': {'precision': args.precision, 'nneigh': int(ff.nlist.nneigh), 'nk': int(nk),
                    'l2': 'flushed (256 MB write) between steps',
                    'parallelism': 'independent replicas' if world > 1 else 'single GPU'},
        'latency_ms': {'p50': float(np.percentile(lat, 50)), 'p99': float(np.percentile(lat, 99))},
        'fp64_evals_per_s': fp64,
        'precision_sweep': sweep,
        'skin_path_evals_per_s': 1.0 / float(np.mean(skin_times)),
        'rebuilds_in_timed_steps': int(nrebuild_timed - nrebuild0),
        'e2e': {'value': e2e, 'unit': 'evals/s', 'h2d_bytes_per_step': natom * 24,
                'd2h_bytes_per_step': natom * 24 + 9 * 8 + 16 * 8},
        'gpu_launches': int(launches),
        'clocks': clk,
        'roofline': roof, 'rooflines': rooflines,
        'peaks_source': pk_src,
    }
    return out, spec


def workload_config(natom):
    """The `config` of both arms' JSON lines (the same workload)."""
    return {'workload': '%s-atom triclinic (82 A, 75 deg) MM3+EI+Ewald, rcut 12 A, skin 1 A, rebuild every step'
                        % format(natom, ','), 'natom': natom}


def precision_sweep(ff, dev, spec, args, step_total, stream, flush, fp64_rate, main_rate):
    """Each precision form against the reference: the error of one
    ForceField.compute(gpos, vtens) at the workload's own positions against
    tests/golden/big_triclinic50000.npz (the reference yaff ForceField.compute
    on the same positions, FP64 on the CPU): energy relative to the total,
    every part's energy relative to the largest part, gradient and virial
    relative RMS; the pair set (SHA-256 of the sorted (a, b, r0, r1, r2)
    keys) for the benchmarked form; and each form's evals/s on the timed
    workload (rebuild every step, L2 flushed)."""
    import hashlib
    import torch
    path = os.path.join(REPO, 'tests', 'golden', 'big_triclinic50000.npz')
    if not os.path.exists(path) or len(spec['pos']) != 50000:
        return None
    ref = np.load(path)
    if not np.array_equal(ref['spec_pos'], spec['pos']):
        return {'error': 'fixture positions differ from the workload'}
    natom = len(spec['pos'])
    e_ref = float(ref['step0_energy'])
    g_ref = ref['step0_gpos']
    v_ref = ref['step0_vtens']
    names = [str(x) for x in ref['step0_parts']]
    pe = ref['step0_part_energy']
    pv = ref['step0_part_vtens']

    def rel_rms(a, b):
        return float(np.sqrt(((a - b) ** 2).mean() / (b ** 2).mean()))

    out = {'reference': 'yaff ForceField.compute, FP64, same positions (tests/golden/big_triclinic50000.npz)',
           'reference_energy': e_ref, 'forms': {}}
    for prec in ('fp64', 'mixed', 'mixed_kahan'):
        dev.set_precision(prec)
        ff.update_pos(spec['pos'])
        ff.nlist.rebuild_next = True
        g = np.zeros((natom, 3))
        v = np.zeros((3, 3))
        e = ff.compute(g, v)
        row = {'energy_rel_err': abs(e - e_ref) / abs(e_ref), 'gpos_rel_rms': rel_rms(g, g_ref),
               'vtens_rel_rms': rel_rms(v, v_ref), 'parts': {}}
        scale = float(np.abs(pe).max())
        for k, nm in enumerate(names):
            part = getattr(ff, 'part_' + nm)
            prow = {'energy_err_rel_largest_part': abs(part.energy - pe[k]) / scale}
            if abs(pv[k]).max() > 0:
                prow['vtens_rel_rms'] = rel_rms(part.vtens, pv[k])
            gp = ref['step0_part_gpos32'][k].astype(np.float64)
            if abs(gp).max() > 0:
                prow['gpos_rel_rms_vs_fp32_copy'] = rel_rms(part.gpos, gp)
            row['parts'][nm] = prow
        row['within_tolerance'] = bool(row['energy_rel_err'] <= (1e-10 if prec == 'fp64' else 1e-6) and
                                       row['gpos_rel_rms'] <= (1e-9 if prec == 'fp64' else 1e-5) and
                                       row['vtens_rel_rms'] <= (1e-9 if prec == 'fp64' else 1e-5))
        if prec == args.precision:
            nb = ff.nlist.neighs
            a = nb['a'].astype(np.int64)
            b = nb['b'].astype(np.int64)
            r = np.stack([nb['r0'], nb['r1'], nb['r2']], 1).astype(np.int64)
            rm = int(np.abs(r).max())
            key = a * natom + b
            for kk in range(3):
                key = key * (2 * rm + 1) + (r[:, kk] + rm)
            order = np.argsort(key, kind='stable')
            keys = np.concatenate([a[order, None], b[order, None], r[order]], 1)
            sha = hashlib.sha256(np.ascontiguousarray(keys, dtype='<i8').tobytes()).hexdigest()
            row['pair_set_equal'] = bool(sha == str(ref['step0_pairs_sha256']) and
                                         len(nb) == int(ref['step0_nneigh']))
            row['nneigh'] = int(len(nb))
        if prec == 'fp64':
            row['evals_per_s'] = fp64_rate
        elif prec == args.precision:
            row['evals_per_s'] = main_rate
        else:
            for s in range(2):
                mask = step_total(s)
            torch.cuda.synchronize()
            tt = []
            for s in range(5):
                flush.fill_(float(s))
                e0 = torch.cuda.Event(enable_timing=True)
                e1 = torch.cuda.Event(enable_timing=True)
                e0.record(stream)
                mask = step_total(s)
                e1.record(stream)
                torch.cuda.synchronize()
                tt.append(e0.elapsed_time(e1) * 1e-3)
            row['evals_per_s'] = 1.0 / float(np.mean(tt))
        out['forms'][prec] = row
    dev.set_precision(args.precision)
    f = out['forms']
    if f['fp64'].get('evals_per_s'):
        out['mixed_over_fp64'] = f['mixed']['evals_per_s'] / f['fp64']['evals_per_s']
    return out


def ff_nk(ff):
    import yaff_gb300
    reci = [p for p in ff.parts if isinstance(p, yaff_gb300.ForcePartEwaldReciprocal)][0]
    g = reci.gmax
    cell = ff.system.cell
    kv = 2 * np.pi * cell.gvecs
    gc2 = (2 * np.pi * reci.gcut) ** 2
    n = 0
    g0, g1, g2 = np.meshgrid(np.arange(-g[0], g[0] + 1), np.arange(-g[1], g[1] + 1), np.arange(0, g[2] + 1),
                             indexing='ij')
    k = g0[..., None] * kv[0] + g1[..., None] * kv[1] + g2[..., None] * kv[2]
    ksq = (k ** 2).sum(-1)
    half = (g2 > 0) | ((g2 == 0) & (g1 > 0)) | ((g2 == 0) & (g1 == 0) & (g0 > 0))
    n = int(((ksq <= gc2) & half).sum())
    return n


def cpu_sample(natom, seconds_budget=20.0):
    """Times the oracle (the reference's algorithm restated in C, FP64, one
    thread) on a bounded decomposition of one force evaluation and scales
    each piece to the full workload: neighbour build on the first M atoms
    (cost ~ M^2), pair terms on those rows, Ewald over a subset of k
    vectors (cost ~ N * nk)."""
    sys.path.insert(0, os.path.join(REPO, 'oracle'))
    import oracle
    from yaff_gb300 import configs
    spec = configs.triclinic_50000() if natom == 50000 else configs.triclinic_mm3_ei(natom=natom)
    N = len(spec['pos'])
    L = oracle.lib()
    cell = oracle.OracleCell(spec['rvecs'])
    rc = spec['rcut'] + spec['skin']
    M = min(N, 16000)
    sub = np.ascontiguousarray(spec['pos'][:M])
    rmax = np.zeros(3, np.int64)
    rows = np.zeros(int(M * 500), oracle.neigh_dtype)
    t0 = time.perf_counter()
    n = L.orc_nlist_build(oracle._p(sub), M, rc, oracle._p(rmax), oracle._p(cell.rvecs), oracle._p(cell.gvecs), 3,
                          0, M, oracle._p(rows), len(rows))
    t_nl = time.perf_counter() - t0
    t_nl_full = t_nl * (N / M) ** 2
    st = np.zeros(0, oracle.scaling_dtype)
    g = np.zeros((N, 3))
    v = np.zeros((3, 3))
    p0, p1 = spec['pair']
    t0 = time.perf_counter()
    L.orc_pair_compute(oracle._p(rows), min(n, len(rows)), oracle._p(st), 0, 1, oracle._p(p0['sigmas']),
                       oracle._p(p0['epsilons']), oracle._p(np.ascontiguousarray(p0['onlypaulis'], np.int32)),
                       None, None, 0.0, 1.0, spec['rcut'], 0, 0.0, oracle._p(g), oracle._p(v))
    L.orc_pair_compute(oracle._p(rows), min(n, len(rows)), oracle._p(st), 0, 2, None, None, None,
                       oracle._p(spec['charges']), oracle._p(np.zeros(N)), spec['ewald']['alpha'], 1.0,
                       spec['rcut'], 0, 0.0, oracle._p(g), oracle._p(v))
    t_pair = time.perf_counter() - t0
    rows_full = 22851584.0 * (N / 50000.0)
    t_pair_full = t_pair * rows_full / max(n, 1)
    # Ewald over a thin slab of k vectors (gmax[0] restricted), scaled by nk
    gmax = np.ceil(spec['ewald']['gcut'] / cell.gspacings - 0.5).astype(np.int64)
    gsub = gmax.copy()
    gsub[0] = 0
    gsub[1] = 5
    work = np.zeros(2 * N)
    t0 = time.perf_counter()
    L.orc_ewald_reci(oracle._p(spec['pos']), N, 0, N, oracle._p(spec['charges']), oracle._p(cell.rvecs),
                     oracle._p(cell.gvecs), cell.volume, spec['ewald']['alpha'], oracle._p(gsub),
                     spec['ewald']['gcut'], 1.0, oracle._p(g), oracle._p(work), oracle._p(v))
    t_ew = time.perf_counter() - t0

    def count_k(gm):
        kv = 2 * np.pi * cell.gvecs
        gc2 = (2 * np.pi * spec['ewald']['gcut']) ** 2
        a, b, c = np.meshgrid(np.arange(-gm[0], gm[0] + 1), np.arange(-gm[1], gm[1] + 1), np.arange(0, gm[2] + 1),
                              indexing='ij')
        k = a[..., None] * kv[0] + b[..., None] * kv[1] + c[..., None] * kv[2]
        half = (c > 0) | ((c == 0) & (b > 0)) | ((c == 0) & (b == 0) & (a > 0))
        return int((((k ** 2).sum(-1) <= gc2) & half).sum())
    nk_sub = count_k(gsub)
    nk_full = count_k(gmax)
    t_ew_full = t_ew * nk_full / max(nk_sub, 1)
    t_eval = t_nl_full + t_pair_full + t_ew_full
    sample = ('oracle (reference algorithm, FP64, 1 thread): nlist on first %d atoms (x(N/M)^2), pair terms on '
              'those %d rows (x rows), Ewald over %d of %d k-vectors (x nk); measured %.1f s' %
              (M, n, nk_sub, nk_full, t_nl + t_pair + t_ew))
    return {'value': 1.0 / t_eval, 'unit': 'evals/s', 'cores': 1, 'kind': 'port', 'sample': sample,
            'seconds_per_eval': t_eval, 'breakdown_s': {'nlist': t_nl_full, 'pair': t_pair_full,
                                                        'ewald_reci': t_ew_full}}


def cpu_whole_eval(natom, threads=None, max_evals=2, budget_s=60.0):
    """Whole force evaluations of the workload with the oracle (the
    reference's algorithm in FP64, yaff_oracle.c) spread over the host cores
    (yaff_oracle_mt.c: the list build, the pair terms and the Ewald
    reciprocal sum on `threads` threads): one untimed evaluation, then up to
    max_evals timed ones (within budget_s), each a full ForceField.compute
    with gradient and virial and a neighbour-list rebuild.  Also returns the
    energy, which equals the reference's to rounding."""
    sys.path.insert(0, os.path.join(REPO, 'oracle'))
    import oracle
    from yaff_gb300 import configs
    spec = configs.triclinic_50000() if natom == 50000 else configs.triclinic_mm3_ei(natom=natom)
    threads = threads or os.cpu_count() or 1
    orc = oracle.OracleForceField(spec, threads=threads)
    n = len(spec['pos'])
    g = np.zeros((n, 3))
    v = np.zeros((3, 3))
    t0 = time.perf_counter()
    e = orc.compute(g, v)
    t_warm = time.perf_counter() - t0
    times = []
    while len(times) < max_evals and sum(times) + t_warm < budget_s:
        orc.rebuild_next = True
        g[:] = 0.0
        v[:] = 0.0
        t0 = time.perf_counter()
        e = orc.compute(g, v)
        times.append(time.perf_counter() - t0)
    return {'seconds_per_eval': float(np.mean(times)), 'evals': len(times), 'cores': threads, 'energy': e,
            'nneigh': int(orc.nneigh)}


def _cpu_serving_request(idx):
    """CPU time of one serving request (50 Verlet steps of 0.5 fs) with the
    oracle as the force field, one thread."""
    import types
    sys.path.insert(0, os.path.join(REPO, 'oracle'))
    from oracle import OracleForceField
    from yaff_gb300.serve import make_workload
    from yaff_gb300.units import femtosecond
    from yaff_gb300.verlet import VerletIntegrator
    r = make_workload(nreq=idx + 1, rate=0.0, seed=2024)[idx]
    t0 = time.perf_counter()
    orc = OracleForceField(r.spec)
    orc.system = types.SimpleNamespace(pos=orc.pos, masses=r.spec['masses'])
    vi = VerletIntegrator(orc, 0.5 * femtosecond, temp0=300.0, rng=np.random.default_rng(r.seed))
    vi.run(r.nsteps)
    return r.natom, time.perf_counter() - t0


def _cpu_mc_trials(seed):
    """CPU time per trial of the MC trial energy with the oracle (the
    reference's algorithm: full force-field evaluations with nlow = nhigh
    plus the structure-factor interaction), one thread, two trials."""
    sys.path.insert(0, os.path.join(REPO, 'oracle'))
    import mc_oracle
    from yaff_gb300 import configs
    work = configs.mc_workload()
    case = {k: work[k] for k in ('framework', 'guest', 'rcut', 'alpha', 'gcut', 'close_contact')}
    rng = np.random.default_rng(100 + seed)
    c = int(rng.integers(0, len(work['chains'])))
    ch, kind, guest, newpos = configs.mc_trial_batch(rng, work, work['chains'], 2, chain_ids=[c])
    t0 = time.perf_counter()
    for t in range(len(ch)):
        mc_oracle.trial_energy(case, list(work['chains'][c]), int(kind[t]), int(guest[t]), newpos[t])
    return (time.perf_counter() - t0) / len(ch)


def cpu_replicas():
    """Replica baselines of the throughput workloads on all host cores: one
    independent single-thread process per core.  Serving: requests of the
    workload with natom <= 1,100 are timed and t = a N^2 + b N is fitted
    (neighbour build and Ewald both grow as N^2 at fixed density), then
    averaged over the workload's natom distribution.  MC: two trials per core."""
    import multiprocessing as mp
    from yaff_gb300.serve import make_workload
    cores = os.cpu_count() or 1
    reqs = make_workload(nreq=4096, rate=0.0, seed=2024)
    small = [i for i, r in enumerate(reqs) if r.natom <= 1100][:cores]
    ctx = mp.get_context('spawn')
    with ctx.Pool(cores) as pool:
        served = pool.map(_cpu_serving_request, small)
        per_trial = pool.map(_cpu_mc_trials, list(range(cores)))
    n = np.array([x[0] for x in served], float)
    t = np.array([x[1] for x in served])
    coef, *_ = np.linalg.lstsq(np.stack([n * n, n], 1), t, rcond=None)
    na = np.array([r.natom for r in reqs], float)
    mean_t = float(coef[0] * (na * na).mean() + coef[1] * na.mean())
    mt = float(np.mean(per_trial))
    return {'cores': cores, 'kind': 'port',
            'serving': {'requests_per_s': cores / mean_t, 'mean_request_s': mean_t,
                        'sample': '%d requests (natom %d-%d) timed with the oracle, t = %.3g N^2 + %.3g N' %
                                  (len(small), int(n.min()), int(n.max()), coef[0], coef[1])},
            'mc': {'trials_per_s': cores / mt, 'seconds_per_trial': mt,
                   'sample': '%d trials on the 2,000-atom framework with the oracle' % (2 * cores)}}


def run_reference(args, world, rank, budget_s=150.0):
    """The reference's algorithm (the oracle port, FP64) on the host cores:
    each step is one whole ForceField.compute(gpos, vtens) of the workload
    with a neighbour-list rebuild, spread over all cores (yaff_oracle_mt.c).
    One untimed warm-up evaluation; then up to --steps timed evaluations,
    stopping early when budget_s is used up -- `steps` is the number that
    actually ran."""
    if rank != 0:
        return None
    sys.path.insert(0, os.path.join(REPO, 'oracle'))
    import oracle
    from yaff_gb300 import configs
    cores = os.cpu_count() or 1
    t_start = time.perf_counter()
    spec = configs.triclinic_50000() if args.natom == 50000 else configs.triclinic_mm3_ei(natom=args.natom)
    n = len(spec['pos'])
    orc = oracle.OracleForceField(spec, threads=cores)
    rng = np.random.default_rng(7)
    pos0 = spec['pos'].copy()
    g = np.zeros((n, 3))
    v = np.zeros((3, 3))
    orc.compute(g, v)
    times = []
    energies = []
    for s in range(args.steps):
        if times and sum(times) + np.mean(times) > budget_s:
            break
        orc.update_pos(pos0 + rng.uniform(-0.05, 0.05, pos0.shape))
        orc.rebuild_next = True
        g[:] = 0.0
        v[:] = 0.0
        t0 = time.perf_counter()
        energies.append(orc.compute(g, v))
        times.append(time.perf_counter() - t0)
    val = len(times) / float(sum(times))
    sample = ('whole force evaluations (neighbour-list rebuild, MM3, EI, Ewald reciprocal / correction / '
              'neutralizing, gradient and virial) of the oracle (the reference algorithm restated in C, FP64) on '
              '%d host threads; %d timed evaluations of %.2f s each after one warm-up' %
              (cores, len(times), float(np.mean(times))))
    return {'metric': 'force evals/s', 'value': val, 'unit': 'evals/s', 'n_gpus': world, 'steps': len(times),
            'steps_requested': args.steps, 'warmup': 1, 'ms_per_step': 1e3 / val, 'higher_is_better': True,
            'scaling': 'weak', 'vs_baseline': None, 'dtype': 'f64',
            'data': 'synthetic (seeded random sequential insertion)', 'impl': 'reference',
            'config': workload_config(args.natom),
            'details': {'precision': 'fp64', 'parallelism': 'one evaluation on %d host threads' % cores},
            'cpu_baseline': {'value': val, 'unit': 'evals/s', 'cores': cores, 'kind': 'port', 'sample': sample},
            'e2e': {'value': val, 'unit': 'evals/s', 'h2d_bytes_per_step': 0, 'd2h_bytes_per_step': 0},
            'nneigh': int(orc.nneigh), 'wall_s': time.perf_counter() - t_start}


def run_serving(args):
    """The serving workload: independent LJ + EI + Ewald systems (natom
    log-uniform in [64, 4000], 0.064 atoms/A^3, rcut 10 A, skin 1 A),
    seeded Poisson arrivals, each request 50 MD steps of 0.5 fs in mixed
    precision, served by the fleet engine (every system in flight stepped
    by one launch per MD phase, continuous admission by free capacity):
    the stated rate, then an arrival-rate sweep up to saturation (all
    requests at t = 0), each with throughput and p50 / p99 latency.  Beside
    it: the per-system-context engine at the stated rate, and the plain FP64
    per-system use (ForceField + host Verlet, one request at a time) on a
    sample of the same requests."""
    from yaff_gb300.fleet import FleetEngine, fleet_bytes
    from yaff_gb300.serve import make_workload, ServingEngine, run_sequential, summarize
    n = args.serving_requests
    caps = dict(max_atoms=1 << 19, max_systems=512, max_k=1 << 21, max_steps=64)
    eng = FleetEngine(chunk=5, **caps)
    eng.run(make_workload(nreq=64, rate=0.0, seed=7), realtime=False)   # warm-up: capture, first builds
    out = {'workload': '%d requests, natom log-uniform [64, 4000], 0.064/A^3, rcut 10 A, skin 1 A, LJ+EI+Ewald, '
                       '50 MD steps of 0.5 fs each, mixed precision, seeded Poisson arrivals' % n,
           'engine': 'fleet: all systems in flight stepped together, 8 launches per MD step (CUDA graph), '
                     'admission every 5 steps by free slots / atom and k ranges',
           'fleet_capacity': dict(caps, bytes=fleet_bytes(caps['max_atoms'], caps['max_systems'], caps['max_k'],
                                                          max_steps=caps['max_steps']))}
    sweep = []
    for rate in (args.serving_rate, 1000.0, 4000.0, 16000.0, 0.0):
        reqs = make_workload(nreq=n, rate=rate, seed=2024)
        eng.peak_inflight = 0
        launches0, steps0 = eng.fleet.launch_count(), eng.steps_run
        wall = eng.run(reqs, realtime=rate > 0)
        row = summarize(reqs, wall)
        row.update({'arrival_rate_per_s': rate if rate > 0 else 'all at t=0 (saturation)',
                    'peak_inflight': eng.peak_inflight,
                    'launches_per_step': (eng.fleet.launch_count() - launches0) / max(1, eng.steps_run - steps0)})
        sweep.append(row)
    out['rate_sweep'] = sweep
    head = sweep[0]
    for k in ('requests', 'errors', 'wall_s', 'requests_per_s', 'atom_steps_per_s', 'latency_p50_ms',
              'latency_p99_ms', 'arrival_rate_per_s'):
        out[k] = head[k]
    out['saturated_requests_per_s'] = sweep[-1]['requests_per_s']
    out['saturated_latency_p99_ms'] = sweep[-1]['latency_p99_ms']
    out['saturated_atom_steps_per_s'] = sweep[-1]['atom_steps_per_s']
    eng.close()
    if args.serving_fleet_only:
        return out
    # the per-system-context engine (one yg_ctx, stream and graph per request)
    nc = min(n, 1024)
    budget = 16 << 30
    ServingEngine(nslots=args.serving_slots, budget_bytes=budget).run(make_workload(nreq=32, rate=0.0, seed=7),
                                                                     realtime=False)
    creq = make_workload(nreq=nc, rate=0.0, seed=2024)
    ceng = ServingEngine(nslots=args.serving_slots, budget_bytes=budget)
    cw = ceng.run(creq, realtime=False)
    cs = summarize(creq, cw)
    out['per_context_engine_saturated'] = {
        'requests': nc, 'slots': args.serving_slots, 'requests_per_s': cs['requests_per_s'],
        'atom_steps_per_s': cs['atom_steps_per_s'], 'latency_p99_ms': cs['latency_p99_ms'],
        'how': 'one context, stream and captured ~45-kernel step per request, all requests at t = 0'}
    # the same engine at the stated arrival rate: below saturation each
    # request runs at the pace of its own context, not of the whole fleet
    rreq = make_workload(nreq=n, rate=args.serving_rate, seed=2024)
    rw = ServingEngine(nslots=args.serving_slots, budget_bytes=budget).run(rreq, realtime=True)
    rs = summarize(rreq, rw)
    out['per_context_engine_at_rate'] = {
        'requests': n, 'arrival_rate_per_s': args.serving_rate, 'slots': args.serving_slots,
        'requests_per_s': rs['requests_per_s'], 'latency_p50_ms': rs['latency_p50_ms'],
        'latency_p99_ms': rs['latency_p99_ms'], 'errors': rs['errors']}
    nseq = min(48, n)
    seq = make_workload(nreq=n, rate=0.0, seed=2024)[:nseq]
    wseq = run_sequential(seq, precision='fp64', mode='api')
    sq = summarize(seq, wseq)
    out['sequential_fp64_api'] = {'requests': nseq, 'requests_per_s': sq['requests_per_s'],
                                  'atom_steps_per_s': sq['atom_steps_per_s'], 'service_p50_ms': sq['service_p50_ms'],
                                  'how': 'ForceField + host VerletIntegrator, FP64, one request at a time'}
    out['saturated_atom_steps_speedup_vs_sequential_fp64'] = out['saturated_atom_steps_per_s'] / sq['atom_steps_per_s']
    return out


def run_nve(args):
    """NVE of the 8,000-molecule flexible water box (24,000 atoms, LJ + EI +
    Ewald + bonds + bends, rcut 10 A, skin 1 A) with the device-resident
    velocity Verlet: 0.5 fs steps, each replayed from a CUDA graph, in the
    mixed and the plain FP64 form.  Both start from the initial velocities of
    tests/golden/md_water24000.npz (the reference's own VerletIntegrator on
    this system) and are compared with the reference over its first steps;
    then --nve-steps timed steps give steps/s, ns/day, the conserved-energy
    drift and fluctuation ratio, and the rebuild count."""
    import torch
    import yaff_gb300
    from yaff_gb300 import configs
    from yaff_gb300.units import femtosecond
    from yaff_gb300.verlet import DeviceVerlet, ConsErrTracker, drift_per_ps
    spec = configs.water_24000()
    natom = len(spec['pos'])
    dt = 0.5 * femtosecond
    n = args.nve_steps
    path = os.path.join(REPO, 'tests', 'golden', 'md_water24000.npz')
    ref = dict(np.load(path)) if os.path.exists(path) else None
    out = {'workload': '8,000 flexible waters (24,000 atoms), LJ+EI+Ewald+bonds+bends, rcut 10 A, skin 1 A, '
                       '0.5 fs velocity Verlet, 300 K initial velocities, device-resident, graph replay',
           'steps': n, 'forms': {}}
    for prec in ('mixed', 'fp64'):
        ff = yaff_gb300.build_forcefield(spec, precision=prec)
        vel0 = ref['vel0'] if ref is not None else None
        dv = DeviceVerlet(ff, dt, vel0=vel0, temp0=300.0, rng=np.random.default_rng(1), max_steps=n + 40,
                          use_graph=True)
        row = {}
        nref = 0
        if ref is not None:
            nref = int(ref['nstep'])
            dv.run(nref)
            pos, vel, log = dv.fetch()
            ep, ek = log[:, 0], log[:, 1]
            escale = float(np.abs(ref['epot']).max())
            row['vs_reference_first_steps'] = {
                'steps': nref,
                'epot_max_abs_err_rel': float(np.abs(ep - ref['epot']).max() / escale),
                'ekin_max_rel_err': float(np.abs(ek - ref['ekin']).max() / np.abs(ref['ekin']).max()),
                'econs_max_abs_err_rel': float(np.abs(ep + ek - ref['econs']).max() / escale),
                'pos_max_abs_err_bohr': float(np.abs(pos - ref['pos_last']).max()),
                'vel_rel_rms': float(np.sqrt(((vel - ref['vel_last']) ** 2).mean() / (ref['vel_last'] ** 2).mean())),
                'reference': 'yaff VerletIntegrator + ForceField, FP64 (tests/golden/md_water24000.npz)'}
        dv.run(40 - nref)  # warm-up: capture and first rebuilds
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        dv.run(n)
        _, _, log = dv.fetch(pos=False, vel=False)
        wall = time.perf_counter() - t0
        log = log[40:]
        econs = log[:, 0] + log[:, 1]
        tr = ConsErrTracker()
        for ep, ek in log:
            tr.update(ek, ep + ek)
        times = dt * np.arange(len(econs))
        sps = n / wall
        row.update({'steps_per_s': sps, 'ns_per_day': sps * 0.5 * 86400 / 1e6,
                    'drift_ha_per_atom_ps': float(drift_per_ps(times, econs, natom)),
                    'cons_err_ratio': float(tr.get()), 'rebuilds': int(dv.nrebuild)})
        out['forms'][prec] = row
        del dv, ff
    f = out['forms']
    out['mixed_over_fp64_steps_per_s'] = f['mixed']['steps_per_s'] / f['fp64']['steps_per_s']
    # headline fields of the mixed form (as before)
    for k in ('steps_per_s', 'ns_per_day', 'drift_ha_per_atom_ps', 'cons_err_ratio', 'rebuilds'):
        out[k] = f['mixed'][k]
    return out


def run_mc(args):
    """MC trial energies: 256 chains on one 2,000-atom framework (0-400 rigid
    waters each), every chain submitting a request of 64 insertion /
    deletion / translation trials; all pending requests go in one launch.
    Host trial arrays in, energies out (H2D + D2H inside the timing)."""
    import torch
    from yaff_gb300 import configs
    from yaff_gb300.mc import MCTrials
    from yaff_gb300.system import Cell
    work = configs.mc_workload()
    cell = Cell(work['framework']['rvecs'])
    nchain = len(work['chains'])
    eng = MCTrials(work['framework'], work['guest'], cell, work['rcut'], work['alpha'], work['gcut'], nchain,
                   work['max_guests'], close_contact=work['close_contact'], precision='mixed')
    for c, g in enumerate(work['chains']):
        eng.set_chain(c, g)
    rng = np.random.default_rng(9)
    batches = [configs.mc_trial_batch(rng, work, work['chains'], 64) for _ in range(args.mc_rounds + 2)]
    out = {'workload': '256 chains x 64 trials per request (1/3 each insertion, deletion, translation of a rigid '
                       'water), 2,000-atom framework in a 30 A cube, 0-400 guests per chain, rcut 12 A, Ewald '
                       'alpha 3.5/rcut, gcut 1.1 alpha, close contact 0.4 A; one launch per 256 requests',
           'trials_per_launch': int(len(batches[0][0])), 'nk': int(eng.prefactors().astype(bool).sum())}
    energies = {}
    for prec in ('mixed', 'fp64'):
        eng.set_precision(prec)
        for b in batches[:2]:
            eng.trials(*b)
        torch.cuda.synchronize()
        lat = []
        for b in batches[2:]:
            t0 = time.perf_counter()
            e = eng.trials(*b)
            lat.append(time.perf_counter() - t0)
        energies[prec] = eng.trials(*batches[2])
        lat = np.array(lat)
        out[prec] = {'trials_per_s': float(len(batches[0][0]) / lat.mean()),
                     'request_latency_ms': {'p50': float(np.percentile(lat, 50) * 1e3),
                                            'p99': float(np.percentile(lat, 99) * 1e3)}}
    ok = np.abs(energies['fp64']) < 1e9
    rel = np.abs(energies['mixed'][ok] - energies['fp64'][ok]) / np.maximum(np.abs(energies['fp64'][ok]), 1e-3)
    out['mixed_vs_fp64_max_rel_err'] = float(rel.max())
    out['close_contact_trials'] = int((~ok).sum())
    out['speedup_mixed_vs_fp64'] = out['mixed']['trials_per_s'] / out['fp64']['trials_per_s']
    eng.destroy()
    return out


def main():
    args = parse()
    world, rank, local = dist_setup()
    if world > 1:
        replicas.init('gloo' if args.impl == 'reference' else 'nccl')
    if args.impl == 'reference':
        out = run_reference(args, world, rank)
        if out is not None:
            print(json.dumps(out))
        return
    out, spec = run_gb300(args, world, rank, local)
    if rank == 0:
        if args.serving_requests > 0 and world == 1:
            out['serving'] = run_serving(args)
        if args.mc_rounds > 0 and world == 1:
            out['mc_trials'] = run_mc(args)
        if args.nve_steps > 0 and world == 1:
            out['nve'] = run_nve(args)
        if not args.no_cpu_baseline and world == 1 and (args.serving_requests > 0 or args.mc_rounds > 0):
            rep = cpu_replicas()
            if 'serving' in out:
                out['serving']['cpu_replicas'] = dict(rep['serving'], cores=rep['cores'], kind=rep['kind'])
            if 'mc_trials' in out:
                out['mc_trials']['cpu_replicas'] = dict(rep['mc'], cores=rep['cores'], kind=rep['kind'])
        if not args.no_cpu_baseline:
            whole = cpu_whole_eval(args.natom)
            one = cpu_sample(args.natom)
            out['cpu_baseline'] = {
                'value': 1.0 / whole['seconds_per_eval'], 'unit': 'evals/s', 'cores': whole['cores'],
                'kind': 'port',
                'sample': '%d whole force evaluation(s) of the workload (rebuild, MM3, EI, Ewald reciprocal / '
                          'correction / neutralizing, gradient and virial) by the oracle on %d host threads, after '
                          'one untimed evaluation' % (whole['evals'], whole['cores']),
                'seconds_per_eval': whole['seconds_per_eval'], 'energy': whole['energy'],
                'single_thread_estimate': {'seconds_per_eval': one['seconds_per_eval'],
                                           'breakdown_s': one['breakdown_s'], 'sample': one['sample']},
                'thread_speedup': one['seconds_per_eval'] / whole['seconds_per_eval']}
        print(json.dumps(out))


if __name__ == '__main__':
    main()
