"""Shared inputs for the tests: seeded systems and comparison helpers."""
from pathlib import Path

import numpy as np

from oracle import md_oracle as O

GOLDEN = Path(__file__).resolve().parent / 'golden'

# LJ fluid of the plain benchmark workload: FCC at rho=0.8442, sigma=eps=1,
# r_cut 2.5 (r_onset 2.0), skin 0.3, dt 0.005, kT 0.722.
LJ_DENSITY = 0.8442
LJ_KT = 0.722
LJ_DT = 0.005
LJ_SKIN = 0.3


def fcc_system(n_cells, seed=0):
    R, L = O.fcc_lattice(n_cells, LJ_DENSITY, 0.05, seed)
    P = O.maxwell_boltzmann(len(R), 3, LJ_KT, seed + 1)
    return R, P, float(L)


def random_box(n, dim, box, seed=0):
    rng = np.random.default_rng(seed)
    return (rng.uniform(0, 1, (n, dim)) * np.asarray(box)).astype(np.float32)


def near_cutoff_pairs(R, box, cutoff, tol=1e-6):
    """Pairs whose f64 distance lies within tol of the list cutoff."""
    R = np.asarray(R, np.float64)
    d = O.displacement(R[:, None, :], R[None, :, :], box)
    r = np.sqrt((d * d).sum(-1))
    i, j = np.nonzero(np.abs(r - cutoff) < tol)
    return set(zip(i.tolist(), j.tolist()))


def lj_spec():
    return O.PairSpec(kind='lj', sigma=1.0, epsilon=1.0, r_onset=2.0, r_cutoff=2.5)
