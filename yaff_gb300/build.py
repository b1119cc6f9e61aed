"""Builds libyaffgb.so (the CUDA kernels and the C ABI) in-tree.

    python -m yaff_gb300.build          # or yaff_gb300.build.build()

Every translation unit in yaff_gb300/csrc is compiled for sm_103a only, in
parallel, and linked into yaff_gb300/_build/libyaffgb.so.  A stamp of the
sources and flags skips the build when nothing changed.
"""
import concurrent.futures
import hashlib
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
REPO = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(BUILD, 'libyaffgb.so')
INCLUDE = os.path.join(REPO, 'include')

ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-ffp-contract=off', '--expt-relaxed-constexpr',
              '-Xptxas', '-warn-spills']


def nvcc():
    path = shutil.which('nvcc')
    if path:
        return path
    cand = '/usr/local/cuda/bin/nvcc'
    if os.path.exists(cand):
        return cand
    raise RuntimeError('nvcc not found')


def sources():
    return sorted(os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith('.cu'))


def _stamp():
    h = hashlib.sha256()
    files = [f for f in sorted(os.listdir(CSRC)) if os.path.isfile(os.path.join(CSRC, f))]
    for f in files + [os.path.join(INCLUDE, 'yaffgb.h')]:
        p = f if os.path.isabs(f) else os.path.join(CSRC, f)
        h.update(p.encode())
        with open(p, 'rb') as fh:
            h.update(fh.read())
    h.update(' '.join(ARCH + NVCC_FLAGS).encode())
    return h.hexdigest()


def build(force=False, verbose=False, extra_flags=()):
    """Compile every .cu for sm_103a and link libyaffgb.so; returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    stamp_file = os.path.join(BUILD, 'stamp')
    stamp = _stamp() + ' '.join(extra_flags)
    if not force and os.path.exists(LIB) and os.path.exists(stamp_file):
        with open(stamp_file) as fh:
            if fh.read() == stamp:
                return LIB
    cc = nvcc()
    objs = []

    def compile_one(src):
        obj = os.path.join(BUILD, os.path.basename(src)[:-3] + '.o')
        cmd = [cc] + ARCH + NVCC_FLAGS + list(extra_flags) + ['-I', INCLUDE, '-c', src, '-o', obj]
        res = subprocess.run(cmd, capture_output=True, text=True)
        if res.returncode != 0:
            raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (src, res.stdout, res.stderr))
        if verbose and (res.stdout or res.stderr):
            sys.stderr.write(res.stdout + res.stderr)
        return obj

    with concurrent.futures.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 2)) as ex:
        objs = list(ex.map(compile_one, sources()))
    tmp = LIB + '.%d.tmp' % os.getpid()
    cmd = [cc] + ARCH + ['-shared', '-o', tmp] + objs + ['-lcudart']
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('link failed:\n%s\n%s' % (res.stdout, res.stderr))
    os.replace(tmp, LIB)
    with open(stamp_file, 'w') as fh:
        fh.write(stamp)
    return LIB


PROBE_SRC = os.path.join(CSRC, 'bench', 'yg_probe.cu')
PROBE_LIB = os.path.join(BUILD, 'libyaffgb_probe.so')


def build_probe():
    """Compile the bench-only throughput probes (csrc/bench/yg_probe.cu) into
    _build/libyaffgb_probe.so; not part of libyaffgb.so.  Returns its path."""
    os.makedirs(BUILD, exist_ok=True)
    deps = [PROBE_SRC, os.path.join(CSRC, 'yg_internal.cuh'), os.path.join(INCLUDE, 'yaffgb.h')]
    if os.path.exists(PROBE_LIB) and os.path.getmtime(PROBE_LIB) >= max(os.path.getmtime(p) for p in deps):
        return PROBE_LIB
    tmp = PROBE_LIB + '.%d.tmp' % os.getpid()
    cmd = [nvcc()] + ARCH + NVCC_FLAGS + ['-I', INCLUDE, '-shared', PROBE_SRC, '-o', tmp, '-lcudart']
    res = subprocess.run(cmd, capture_output=True, text=True)
    if res.returncode != 0:
        raise RuntimeError('nvcc failed for %s:\n%s\n%s' % (PROBE_SRC, res.stdout, res.stderr))
    os.replace(tmp, PROBE_LIB)
    return PROBE_LIB


if __name__ == '__main__':
    print(build(force='--force' in sys.argv, verbose=True))
    print(build_probe())
