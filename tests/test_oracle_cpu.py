"""The C/OpenMP float32 restatement used as the timed CPU baseline
(oracle/md_cpu.c) against the FP64 oracle: NVE (simulate.py:227-243) and
Nose-Hoover NVT (simulate.py:649-667) on the LJ benchmark's lattice start.
CPU only (gcc + OpenMP)."""
import ctypes

import numpy as np
import pytest

from oracle import md_oracle as O
from tests.helpers import fcc_system

fp = ctypes.POINTER(ctypes.c_float)
dp = ctypes.POINTER(ctypes.c_double)


@pytest.fixture(scope='module')
def lib():
    from oracle import build
    L = ctypes.CDLL(str(build.build()))
    L.md_cpu_run.argtypes = [fp, fp, ctypes.c_int, ctypes.c_float, ctypes.c_float, ctypes.c_float,
                             ctypes.c_float, ctypes.c_float, ctypes.c_int, ctypes.c_int,
                             ctypes.c_int]
    L.md_cpu_run_nvt.argtypes = L.md_cpu_run.argtypes + [ctypes.c_double, ctypes.c_double,
                                                         ctypes.c_int, ctypes.c_int, ctypes.c_int,
                                                         dp]
    return L


def _oracle_run(R, P, L, steps, nvt=None):
    box = np.full(3, L)
    nl = O.NeighborListOracle(box, 2.5, 0.3, fmt=O.DENSE)
    h = {'nb': nl.allocate(R)}

    def fn(X):
        h['nb'] = nl.update(X, h['nb'])
        return O.pair_energy_forces(O.PairSpec(kind='lj'), X, h['nb'].idx, O.DENSE, box)[1]
    X, Pd = R.astype(np.float64), P.astype(np.float64)
    F = fn(X)
    c = None
    if nvt:
        kT, tau = nvt
        c = O.nhc_init(3 * len(R), O.kinetic_energy(Pd), kT, tau, 5)
    for _ in range(steps):
        if nvt:
            X, Pd, F, c = O.nvt_nose_hoover_step(fn, X, Pd, F, 1.0, c, 0.005, nvt[0], box)
        else:
            X, Pd, F = O.velocity_verlet(fn, X, Pd, F, 1.0, 0.005, box)
    return X, Pd, c


def test_c_baseline_nve_matches_oracle(lib):
    R, P, L = fcc_system(6)
    x, p = R.astype(np.float32).copy(), P.astype(np.float32).copy()
    steps = 30
    rb = lib.md_cpu_run(x.ctypes.data_as(fp), p.ctypes.data_as(fp), len(x), float(L), 2.0, 2.5,
                        0.3, 0.005, 128, steps, 2)
    assert rb >= 0
    X, Pd, _ = _oracle_run(R, P, L, steps)
    assert np.abs(O.displacement(x, X, np.full(3, L))).max() < 1e-4
    assert np.abs(p - Pd).max() < 1e-3


def test_c_baseline_nvt_matches_oracle(lib):
    R, P, L = fcc_system(6, 2)
    x, p = R.astype(np.float32).copy(), P.astype(np.float32).copy()
    steps, kT, tau = 30, 0.722, 0.5
    chain = np.zeros(16)
    rb = lib.md_cpu_run_nvt(x.ctypes.data_as(fp), p.ctypes.data_as(fp), len(x), float(L), 2.0, 2.5,
                            0.3, 0.005, 128, steps, 2, kT, tau, 5, 2, 3,
                            chain.ctypes.data_as(dp))
    assert rb >= 0
    X, Pd, c = _oracle_run(R, P, L, steps, nvt=(kT, tau))
    assert np.abs(O.displacement(x, X, np.full(3, L))).max() < 1e-4
    assert np.abs(p - Pd).max() < 1e-3
    np.testing.assert_allclose(chain[5:10], c.p_xi, rtol=1e-3, atol=1e-4)
    np.testing.assert_allclose(chain[:5], c.xi, rtol=1e-3, atol=1e-6)
    assert abs(chain[15] - c.KE) <= 1e-5 * c.KE
