"""Build libcommit_gb300.so (sm_103a) in-tree with nvcc.

Each .cu file is compiled to an object in commit_gb300/_build (in parallel), then linked
into commit_gb300/libcommit_gb300.so with the CUDA runtime linked statically.  Objects
are rebuilt when a source or header is newer or the machine architecture changed.
"""
from __future__ import annotations

import concurrent.futures as cf
import glob
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, 'csrc')
BUILD = os.path.join(HERE, '_build')
LIB = os.path.join(HERE, 'libcommit_gb300.so')
STAMP = os.path.join(BUILD, 'arch.txt')

GENCODE = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-lineinfo', '-std=c++17', '-Xcompiler', '-fPIC', '-Xcompiler', '-O2',
              # host code: no fused multiply-adds, so the solver's host-side FP64 decisions are the
              # same bits on every host architecture (and equal to the graph mode's device ones)
              '-Xcompiler', '-ffp-contract=off',
              '--expt-relaxed-constexpr', '-diag-suppress', '128', '-I', os.path.join(ROOT, 'include')]


# per-file extra flags: the voxeliser reproduces the reference's FP64 geometry operation
# by operation, so no multiply-add may be fused there
FILE_FLAGS = {'trk2dict.cu': ['-fmad=false']}


def nvcc() -> str:
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and os.path.exists(cand):
            return cand
    raise RuntimeError('nvcc not found')


def _headers():
    return glob.glob(os.path.join(CSRC, '*.cuh')) + glob.glob(os.path.join(ROOT, 'include', '*.h'))


def _stale(obj: str, src: str, headers: list) -> bool:
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    return any(os.path.getmtime(p) > t for p in [src] + headers)


def build(verbose: bool = False, jobs: int | None = None) -> str:
    os.makedirs(BUILD, exist_ok=True)
    arch = platform.machine()
    if not os.path.exists(STAMP) or open(STAMP).read().strip() != arch:
        for o in glob.glob(os.path.join(BUILD, '*.o')):
            os.remove(o)
        if os.path.exists(LIB):
            os.remove(LIB)
    headers = _headers()
    srcs = sorted(glob.glob(os.path.join(CSRC, '*.cu')))
    objs = [os.path.join(BUILD, os.path.basename(s)[:-3] + '.o') for s in srcs]
    todo = [(s, o) for s, o in zip(srcs, objs) if _stale(o, s, headers)]
    nv = nvcc()

    def compile_one(so):
        s, o = so
        cmd = [nv] + GENCODE + NVCC_FLAGS + FILE_FLAGS.get(os.path.basename(s), []) + ['-c', s, '-o', o + '.tmp']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError(f'nvcc failed on {os.path.basename(s)}:\n{r.stderr[-4000:]}')
        os.replace(o + '.tmp', o)
        return s

    if todo:
        n = jobs or min(len(todo), max(1, os.cpu_count() or 1))
        with cf.ThreadPoolExecutor(max_workers=n) as ex:
            for s in ex.map(compile_one, todo):
                if verbose:
                    print('compiled', os.path.basename(s), flush=True)
    if todo or not os.path.exists(LIB):
        cmd = [nv] + GENCODE + ['-shared', '-cudart', 'static', '-o', LIB + '.tmp'] + objs
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError('link failed:\n' + r.stderr[-4000:])
        os.replace(LIB + '.tmp', LIB)
        with open(STAMP, 'w') as f:
            f.write(arch)
    return LIB


if __name__ == '__main__':
    print(build(verbose=True))
    sys.exit(0)
