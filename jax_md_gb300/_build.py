"""Builds the sm_103a shared library ``libjaxmd_gb300.so`` in-tree.

Plain nvcc, one translation unit per kernel family compiled in parallel, no
CMake.  The library is the C ABI declared in ``include/jax_md_gb300.h``.
"""
from __future__ import annotations

import concurrent.futures as cf
import os
import shutil
import subprocess
import sys
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
CSRC = PKG / 'csrc'
BUILD = PKG / '_build'
LIB = PKG / 'libjaxmd_gb300.so'

SOURCES = ['api.cu', 'nlist.cu', 'pair.cu', 'integrate.cu', 'fused.cu', 'tiled.cu', 'segment.cu',
           'adjoint.cu', 'batched.cu', 'engine.cu']
ARCH = ['-gencode', 'arch=compute_103a,code=sm_103a']
NVCC_FLAGS = ['-O3', '-std=c++17', '-lineinfo', '-Xcompiler', '-fPIC', '--expt-relaxed-constexpr',
              '-Xptxas', '-warn-spills']


def nvcc() -> str:
    for cand in (os.environ.get('NVCC'), shutil.which('nvcc'), '/usr/local/cuda/bin/nvcc'):
        if cand and Path(cand).exists():
            return cand
    raise RuntimeError('nvcc not found: the CUDA toolkit is required to build jax_md_gb300')


def _stale(target: Path, deps) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(Path(d).stat().st_mtime > t for d in deps)


def build(verbose: bool = False, force: bool = False) -> Path:
    BUILD.mkdir(exist_ok=True)
    headers = list(CSRC.glob('*.cuh')) + [ROOT / 'include' / 'jax_md_gb300.h']
    srcs = [CSRC / s for s in SOURCES if (CSRC / s).exists()]
    objs = []
    jobs = []
    for s in srcs:
        o = BUILD / (s.stem + '.o')
        objs.append(o)
        if force or _stale(o, [s] + headers):
            cmd = [nvcc(), *ARCH, *NVCC_FLAGS, '-c', str(s), '-o', str(o)]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        return cmd, r

    with cf.ThreadPoolExecutor(max_workers=min(8, max(1, len(jobs)))) as ex:
        for cmd, r in ex.map(run, jobs):
            if verbose or r.returncode != 0:
                sys.stderr.write(' '.join(cmd) + '\n' + r.stdout + r.stderr)
            if r.returncode != 0:
                raise RuntimeError(f'nvcc failed on {cmd[-3]}')
    if force or jobs or _stale(LIB, objs):
        cmd = [nvcc(), *ARCH, '-shared', '-o', str(LIB), *map(str, objs), '-lcudart']
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            sys.stderr.write(r.stdout + r.stderr)
            raise RuntimeError('linking libjaxmd_gb300.so failed')
    return LIB


if __name__ == '__main__':
    build(verbose='-v' in sys.argv, force='-f' in sys.argv)
    print(LIB)
