"""Builds the oracle's C baseline (oracle/_build/libmdcpu.so) with gcc + OpenMP.

Test / baseline infrastructure: only tests, smoke() and bench.py's CPU legs
load it.  The reference (Python/JAX) has no compiled sources, so there is no
oracle/_ref build.
"""
import subprocess
from pathlib import Path

HERE = Path(__file__).resolve().parent
OUT = HERE / '_build' / 'libmdcpu.so'


def build() -> Path:
    OUT.parent.mkdir(exist_ok=True)
    src = HERE / 'md_cpu.c'
    if OUT.exists() and OUT.stat().st_mtime >= src.stat().st_mtime:
        return OUT
    cmd = ['gcc', '-O3', '-fopenmp', '-shared', '-fPIC', '-o', str(OUT), str(src), '-lm']
    subprocess.run(cmd, check=True)
    return OUT


if __name__ == '__main__':
    print(build())
