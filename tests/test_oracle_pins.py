"""Pins the FP64 oracle to the reference's golden fixtures and known answers.

CPU only.  Each case cites the reference test it restates.
"""
import math

import numpy as np
import pytest

from oracle import md_oracle as O
from tests.helpers import GOLDEN, fcc_system, random_box


def test_lammps_lj_energy_and_stress():
    """tests/quantity_test.py:436-455: truncated LJ at 2.5, tol 5e-5."""
    g = np.load(GOLDEN / 'lammps_lj_stress.npz')
    box = float(g['box'])
    R = g['fractional_position'] * box
    V = g['velocity']
    spec = O.PairSpec(kind='lj_truncated', r_cutoff=2.5)
    E, F, W = O.all_pairs_energy_forces(spec, R, np.full(3, box))
    assert abs(E / len(R) - g['energy_per_atom']) < 5e-5
    S = O.stress(W, V, 1.0, box ** 3)
    np.testing.assert_allclose(S, g['stress'], atol=5e-5, rtol=5e-5)


def test_jammed_soft_sphere_pressure_and_energy():
    """tests/quantity_test.py:134-150 (pressure, f64 tol 1e-7) + the stored energy."""
    g = np.load(GOLDEN / 'jammed_soft_sphere_2d.npz')
    L = np.diag(g['box'])
    spec = O.PairSpec(kind='soft_sphere', sigma=g['sigma'], epsilon=1.0, alpha=2.0,
                      species=g['species'])
    E, F, W = O.all_pairs_energy_forces(spec, g['real_position'], L)
    P = O.pressure(W, 0.0, 2, np.prod(L))
    assert abs(P - g['pressure']) < 1e-7
    assert abs(E - g['energy']) < 1e-10


def test_lj_minimum():
    """tests/energy_test.py:325-342: U(2^(1/6) sigma) = -eps, U' = 0."""
    for sigma, eps in [(1.0, 1.0), (0.5, 2.0), (1.3, 0.7)]:
        r = np.array([2 ** (1 / 6) * sigma])
        U, dU, _ = O.lennard_jones(r, sigma, eps)
        assert abs(U[0] + eps) < 1e-12
        assert abs(dU[0]) < 1e-10


def test_soft_sphere_known_values():
    """tests/energy_test.py:284-312."""
    for alpha in (2.0, 2.5, 3.0):
        sigma, eps = 1.3, 0.8
        U, dU, _ = O.soft_sphere(np.array([0.0, sigma, 2 * sigma]), sigma, eps, alpha)
        assert abs(U[0] - eps / alpha) < 1e-12
        assert U[1] == 0.0 and U[2] == 0.0
        assert dU[2] == 0.0
        if alpha > 2:
            assert abs(dU[1]) < 1e-12


def test_multiplicative_cutoff_regions():
    """tests/energy_test.py:533-562: identity below r_onset, zero beyond r_cutoff, C1."""
    r = np.linspace(0.5, 3.0, 1001)
    S, dS, _ = O.multiplicative_cutoff(r, 2.0, 2.5)
    assert np.all(S[r < 2.0] == 1.0)
    assert np.all(S[r >= 2.5] == 0.0)
    # continuity of S and S' at both ends
    for r0 in (2.0, 2.5):
        s_l, ds_l, _ = O.multiplicative_cutoff(np.array([r0 - 1e-7]), 2.0, 2.5)
        s_r, ds_r, _ = O.multiplicative_cutoff(np.array([r0 + 1e-7]), 2.0, 2.5)
        assert abs(s_l - s_r) < 1e-6 and abs(ds_l - ds_r) < 1e-5


def test_oracle_second_derivative_matches_fd():
    spec = O.PairSpec(kind='lj')
    r = np.linspace(0.9, 2.6, 301)
    h = 1e-6
    _, dU, d2U = O.pair_terms(spec, r)
    _, dUp, _ = O.pair_terms(spec, r + h)
    _, dUm, _ = O.pair_terms(spec, r - h)
    fd = (dUp - dUm) / (2 * h)
    mask = (np.abs(r - 2.0) > 1e-3) & (np.abs(r - 2.5) > 1e-3)
    np.testing.assert_allclose(d2U[mask], fd[mask], rtol=1e-5, atol=1e-5)


def test_cell_list_emplace_2d():
    """tests/partition_test.py:61-98: slot rule hash*cap + (rank mod cap)."""
    R = np.array([[0.25, 0.25], [8.5, 1.95], [8.1, 1.5], [3.7, 7.9]], np.float32)
    box = np.array([8.65, 8.0], np.float32)
    cap = O.estimate_cell_capacity(R, box, 1.0, 1.25, 2)
    cl = O.cell_list(R, box, 1.0, cap)
    cps = cl.cells_per_side
    ids = cl.id_buffer.reshape(cps[1], cps[0], cap)
    assert ids[0, 0, 0] == 0
    assert ids[1, 7, 1] == 1   # the reference indexes [1, 8, 1] and JAX clamps 8 -> 7
    assert ids[1, 7, 0] == 2
    assert ids[7, 3, 1] == 3


@pytest.mark.parametrize('dim', [2, 3])
def test_oracle_neighbor_list_matches_all_pairs(dim):
    """tests/partition_test.py:203-257: neighbour sets == brute force, rectangular box."""
    box = np.array([9.0, 3.25] if dim == 2 else [9.0, 4.0, 7.25], np.float32)
    R = random_box(400, dim, box, seed=3)
    nl = O.NeighborListOracle(box, 1.23 / 2, 0.0, fmt=O.DENSE)  # 3 cells on the short side
    nb = nl.allocate(R)
    assert nb.use_cell_list
    sets = O.neighbor_sets(nb, len(R))
    d = O.displacement(R[:, None], R[None], box)
    r2 = (d * d).sum(-1)
    for i in range(len(R)):
        brute = sorted(int(j) for j in np.nonzero(r2[i] < nl.cutoff_sq)[0] if j != i)
        assert sets[i] == brute


@pytest.mark.parametrize('r_cut,dc,cm', [(0.12, True, 1.5), (0.25, False, 1.5),
                                         (0.31, False, 1.5), (0.31, False, 1.0)])
@pytest.mark.parametrize('mask_self', [False, True])
@pytest.mark.parametrize('fmt', [O.DENSE, O.SPARSE, O.ORDERED_SPARSE])
def test_capacity_shapes(r_cut, dc, cm, mask_self, fmt):
    """tests/partition_test.py:489-546 (issue 191): 20 atoms at one point."""
    if fmt == O.DENSE:
        want = (20, 19) if mask_self else (20, 20)
    elif fmt == O.SPARSE:
        want = (2, 20 * 19) if mask_self else (2, 400)
    else:
        want = (2, 20 * 19 // 2)
    R = np.full((20, 3), 0.5, np.float32)
    nl = O.NeighborListOracle(np.ones(3), r_cut, 0.1 * r_cut, capacity_multiplier=cm,
                              disable_cell_list=dc, mask_self=mask_self, fmt=fmt)
    nb = nl.allocate(R)
    assert not O.did_buffer_overflow(nb.error)
    assert nb.idx.shape == want
    nb2 = nl.update(R + np.float32(0.1), nb)
    assert not O.did_buffer_overflow(nb2.error)
    assert nb2.idx.shape == want


def test_overflow_on_collapse():
    """tests/partition_test.py:363-401: free space, two points collapse -> overflow."""
    R = np.array([[20.0, 20.0], [30.0, 30.0], [40.0, 40.0], [50.0, 50.0]], np.float32)
    nl = O.NeighborListOracle(100.0, 3.0, 0.0, periodic=False)
    nb = nl.allocate(R)
    assert not O.did_buffer_overflow(nb.error)
    R2 = R.copy()
    R2[1] = R2[0]
    nb2 = nl.update(R2, nb)
    assert O.did_buffer_overflow(nb2.error)


def test_nhc_invariant_drift_small():
    """simulate_test.py:264-304 style: NVT invariant conserved (oracle, small system)."""
    R, P, L = fcc_system(3)
    box = np.full(3, L)
    spec = O.PairSpec(kind='lj')
    nl = O.NeighborListOracle(box, 2.5, 0.3)
    nb = nl.allocate(R)
    def fn(X):
        return O.pair_energy_forces(spec, X, nb.idx, O.DENSE, box)[1]
    R = R.astype(np.float64)
    P = P.astype(np.float64)
    F = fn(R)
    c = O.nhc_init(R.size, O.kinetic_energy(P), 0.722, 0.5, 5)
    H0 = O.nvt_invariant(O.pair_energy_forces(spec, R, nb.idx, O.DENSE, box)[0], P, 1.0, c, 0.722)
    for _ in range(100):
        R, P, F, c = O.nvt_nose_hoover_step(fn, R, P, F, 1.0, c, 0.005, 0.722, box)
    H1 = O.nvt_invariant(O.pair_energy_forces(spec, R, nb.idx, O.DENSE, box)[0], P, 1.0, c, 0.722)
    assert abs(H1 - H0) / len(R) < 5e-4


def test_morse_minimum_and_scaled_form():
    """tests/energy_test.py:479-520: U(sigma) = -eps with zero slope for random
    (sigma, eps, alpha); at r = a / alpha + sigma, U / eps = (1 - e^-a)^2 - 1
    whatever sigma, eps and alpha are."""
    rng = np.random.default_rng(17)
    for _ in range(16):
        sig, eps, alp = rng.uniform(0.0, 3.0), rng.uniform(0.0, 4.0), rng.uniform(1.0, 30.0)
        U, dU, _ = O.morse(np.array([sig]), sig, eps, alp)
        assert abs(U[0] + eps) <= 1e-12 * max(1.0, eps) and abs(dU[0]) <= 1e-12
    for _ in range(16):
        sig, eps, alp = rng.uniform(0.0, 3.0), rng.uniform(0.1, 4.0), rng.uniform(1.0, 30.0)
        a = np.linspace(max(-2.5, -alp * sig), 8.0, 100)
        U, _, _ = O.morse(a / alp + sig, sig, eps, alp)
        np.testing.assert_allclose(U / eps, (1.0 - np.exp(-a)) ** 2 - 1.0, rtol=1e-10, atol=1e-12)


def test_morse_derivatives_match_fd():
    """U' and U'' of the cut-off Morse pair (absolute radii 2.0 / 2.5) against
    central differences, away from the two switch radii."""
    spec = O.PairSpec(kind='morse', sigma=1.1, epsilon=5.0, alpha=5.0)
    r = np.linspace(0.8, 2.6, 361)
    h = 1e-6
    U, dU, d2U = O.pair_terms(spec, r)
    Up, dUp, _ = O.pair_terms(spec, r + h)
    Um, dUm, _ = O.pair_terms(spec, r - h)
    mask = (np.abs(r - 2.0) > 1e-3) & (np.abs(r - 2.5) > 1e-3)
    np.testing.assert_allclose(dU[mask], ((Up - Um) / (2 * h))[mask], rtol=1e-5, atol=1e-6)
    np.testing.assert_allclose(d2U[mask], ((dUp - dUm) / (2 * h))[mask], rtol=1e-5, atol=1e-5)
    assert np.all(U[r >= 2.5] == 0.0) and np.all(dU[r >= 2.5] == 0.0)
    bare, _, _ = O.morse(r, 1.1, 5.0, 5.0)
    np.testing.assert_array_equal(U[r < 2.0], bare[r < 2.0])


@pytest.mark.parametrize('fmt', [O.DENSE, O.SPARSE, O.ORDERED_SPARSE])
def test_morse_neighbor_list_matches_all_pairs(fmt):
    """tests/energy_test.py:647-700, 852-875: the Morse neighbour-list energy
    and forces equal the all-pairs ones (morse_pair) in every format."""
    box = np.array([6.0, 6.0, 6.0], np.float32)
    R = random_box(150, 3, box, seed=5)
    spec = O.PairSpec(kind='morse', sigma=1.0, epsilon=5.0, alpha=5.0)
    E0, F0, W0 = O.all_pairs_energy_forces(spec, R, box)
    nl = O.NeighborListOracle(box, 2.5, 0.5, fmt=fmt)
    E, F, W = O.pair_energy_forces(spec, R, nl.allocate(R).idx, fmt, box)
    assert abs(E - E0) <= 1e-10 * max(1.0, abs(E0))
    np.testing.assert_allclose(F, F0, rtol=1e-10, atol=1e-10)
    np.testing.assert_allclose(W, W0, rtol=1e-10, atol=1e-10)


class _WithKwargs:
    """A space whose displacement always passes box= / new_box= keywords."""

    def __init__(self, sp, **kw):
        self.sp, self.kw = sp, kw

    def displacement(self, Ra, Rb):
        return self.sp.displacement(Ra, Rb, **self.kw)


@pytest.mark.parametrize('dim', [2, 3])
def test_periodic_general_diagonal_matches_periodic(dim):
    """tests/space_test.py:302-350: a diagonal periodic_general box gives the
    displacements of space.periodic on scaled positions, and its shift
    times the sides gives periodic's shift."""
    rng = np.random.default_rng(21)
    for _ in range(10):
        sides = 10.0 * rng.uniform(0.05, 1.0, dim)
        R = rng.uniform(0.0, 1.0, (10, dim))
        dR = rng.standard_normal((10, dim))
        g = O.PeriodicGeneral(np.diag(sides))
        d_per = O.displacement(R[:, None] * sides, R[None] * sides, sides)
        np.testing.assert_allclose(g.displacement(R[:, None], R[None]), d_per, atol=1e-13)
        np.testing.assert_allclose(O.periodic_shift(sides, R * sides, dR), g.shift(R, dR) * sides,
                                   atol=1e-12)


@pytest.mark.parametrize('dim', [2, 3])
def test_periodic_general_wrapped_vs_unwrapped(dim):
    """tests/space_test.py:456-500: wrapping positions back into the cell does
    not change displacements (T = I + dT + dT^T)."""
    rng = np.random.default_rng(22)
    for _ in range(10):
        dT = rng.standard_normal((dim, dim))
        T = np.eye(dim) + dT + dT.T
        if abs(np.linalg.det(T)) < 0.1:
            continue
        R0 = rng.uniform(0.0, 1.0, (10, dim))
        R, Ru = R0.copy(), R0.copy()
        g, gu = O.PeriodicGeneral(T), O.PeriodicGeneral(T, wrapped=False)
        for _ in range(10):
            dR = rng.standard_normal((10, dim))
            R, Ru = g.shift(R, dR), gu.shift(Ru, dR)
            np.testing.assert_allclose(g.displacement(R[:, None], R0[None]),
                                       g.displacement(Ru[:, None], R0[None]), atol=1e-9)
        assert np.all((R >= 0) & (R < 1)) and not np.all((Ru > 0) & (Ru < 1))


def _general_systems(dim, box_format, seed=0):
    """tests/space_test.py:48-71: 16 soft spheres at unit density in a
    periodic box given as a scalar, a vector or a matrix, in the three
    parameterisations (periodic, periodic_general fractional and real)."""
    n = 16
    L = n ** (1.0 / dim)
    box = {'scalar': L, 'vector': np.full(dim, L), 'matrix': np.eye(dim) * L}[box_format]
    R_f = np.random.default_rng(seed).uniform(0.0, 1.0, (n, dim))
    R = O.transform(box, R_f)
    side = np.diag(box) if box_format == 'matrix' else box
    return R_f, R, box, side


@pytest.mark.parametrize('box_format', ['scalar', 'vector', 'matrix'])
@pytest.mark.parametrize('dim', [2, 3])
def test_periodic_general_energy_force_shift(dim, box_format):
    """tests/space_test.py:509-575: the three parameterisations give the same
    soft-sphere energy and the same real-space forces (the reference's
    transform JVP keeps gradients in real space), and shifting by those
    forces gives the same positions."""
    R_f, R, box, side = _general_systems(dim, box_format)
    spec = O.PairSpec(kind='soft_sphere')
    gf = O.PeriodicGeneral(box)
    gr = O.PeriodicGeneral(box, fractional_coordinates=False)
    E, F, _ = O.all_pairs_energy_forces(spec, R, np.broadcast_to(side, (dim,)))
    E_f, F_f, _ = O.all_pairs_energy_forces(spec, R_f, gf)
    E_r, F_r, _ = O.all_pairs_energy_forces(spec, R, gr)
    assert E > 0 and abs(E - E_f) < 1e-12 and abs(E - E_r) < 1e-12
    np.testing.assert_allclose(F, F_f, atol=1e-12)
    np.testing.assert_allclose(F, F_r, atol=1e-12)
    new = O.periodic_shift(np.broadcast_to(side, (dim,)), R, F)
    np.testing.assert_allclose(new, O.transform(box, gf.shift(R_f, F_f)), atol=1e-12)
    np.testing.assert_allclose(new, gr.shift(R, F_r), atol=1e-12)


@pytest.mark.parametrize('box_format', ['scalar', 'vector', 'matrix'])
@pytest.mark.parametrize('dim', [2, 3])
def test_periodic_general_deform(dim, box_format):
    """tests/space_test.py:577-598: a deformed box passed as box= to the
    fractional space equals new_box= to the real-coordinate space."""
    R_f, R, box, _ = _general_systems(dim, box_format)
    spec = O.PairSpec(kind='soft_sphere')
    deformed = np.asarray(box) * 0.9
    E_f = O.all_pairs_energy_forces(spec, R_f, _WithKwargs(O.PeriodicGeneral(box), box=deformed))[0]
    E_r = O.all_pairs_energy_forces(
        spec, R, _WithKwargs(O.PeriodicGeneral(box, fractional_coordinates=False),
                             new_box=deformed))[0]
    assert E_f > 0 and abs(E_f - E_r) < 1e-12


def test_periodic_general_triclinic_parameterisations_agree():
    """An upper-triangular (triclinic) cell: fractional and real coordinates
    give the same LJ energy and forces, and a pure shear of the cell changes
    the energy (the tilt enters the displacement)."""
    T = np.array([[6.0, 1.2, 0.7], [0.0, 5.5, -0.9], [0.0, 0.0, 6.5]])
    R_f = np.random.default_rng(4).uniform(0.0, 1.0, (60, 3))
    spec = O.PairSpec(kind='lj_truncated', r_cutoff=2.5)
    E_f, F_f, _ = O.all_pairs_energy_forces(spec, R_f, O.PeriodicGeneral(T))
    E_r, F_r, _ = O.all_pairs_energy_forces(spec, O.transform(T, R_f),
                                            O.PeriodicGeneral(T, fractional_coordinates=False))
    assert abs(E_f - E_r) <= 1e-10 * abs(E_f)
    np.testing.assert_allclose(F_f, F_r, rtol=1e-9, atol=1e-9)
    E_0 = O.all_pairs_energy_forces(spec, R_f, O.PeriodicGeneral(np.diag(np.diag(T))))[0]
    assert abs(E_f - E_0) > 1e-6 * abs(E_0)


@pytest.mark.parametrize('fmt', [O.DENSE, O.SPARSE, O.ORDERED_SPARSE])
@pytest.mark.parametrize('dim', [2, 3])
def test_per_particle_params_neighbor_list_matches_all_pairs(dim, fmt):
    """tests/smap_test.py:1308-1340: per-particle sigma_i ~ U[0.5, 1.5]
    combined as 0.5 (sigma_i + sigma_j); a list with cutoff max sigma gives
    the all-pairs energy, in every format."""
    rng = np.random.default_rng(31 + dim)
    n = 120
    L = 2.0 * n ** (1.0 / dim)
    box = np.full(dim, L)
    R = rng.uniform(0.0, L, (n, dim))
    sig = rng.uniform(0.5, 1.5, n)
    spec = O.PairSpec(kind='soft_sphere', sigma=sig)
    E0, F0, _ = O.all_pairs_energy_forces(spec, R, box)
    nl = O.NeighborListOracle(box, float(sig.max()), 0.0, fmt=fmt)
    E, F, _ = O.pair_energy_forces(spec, R, nl.allocate(R).idx, fmt, box)
    assert E0 > 0 and abs(E - E0) <= 1e-12 * E0
    np.testing.assert_allclose(F, F0, atol=1e-12)


def test_per_particle_params_combinator_and_uniform_arrays():
    """The pair parameter is the mean of the two atoms' values; uniform
    per-particle arrays reproduce the scalar parameters (LJ, radii from
    max sigma)."""
    R = np.array([[0.0, 0.0, 0.0], [1.1, 0.0, 0.0]])
    spec = O.PairSpec(kind='lj', sigma=np.array([0.9, 1.3]), epsilon=np.array([1.0, 2.0]))
    E = O.all_pairs_energy_forces(spec, R)[0]
    U, _, _ = O.pair_terms(O.PairSpec(kind='lj', sigma=1.1, epsilon=1.5, r_onset=2.0 * 1.3 / 1.1,
                                      r_cutoff=2.5 * 1.3 / 1.1), np.array([1.1]))
    assert abs(E - U[0]) < 1e-12
    box = np.full(3, 7.0)
    Rb = random_box(80, 3, box.astype(np.float32), seed=2)
    a = O.all_pairs_energy_forces(O.PairSpec(kind='lj', sigma=np.full(80, 1.05),
                                             epsilon=np.full(80, 0.8)), Rb, box)
    b = O.all_pairs_energy_forces(O.PairSpec(kind='lj', sigma=1.05, epsilon=0.8), Rb, box)
    assert abs(a[0] - b[0]) <= 1e-12 * abs(b[0])
    np.testing.assert_allclose(a[1], b[1], atol=1e-10)


def test_langevin_harmonic_matches_theory():
    """tests/simulate_test.py:872-915: 200,000 independent 1-D oscillators
    (alpha 1, mass 3, gamma 3, kT 0.25, dt 1e-4) from x = 1 and thermal
    momenta; after 1000 BAOAB steps the mean position and the momentum
    autocorrelation follow the overdamped-oscillator solution.  The
    reference's 1e-3 holds for its own random stream; with another stream the
    bound is four standard errors of the sample mean (SE ~ 2.4e-3 for the
    autocorrelation) plus 1e-3 relative."""
    alpha, mass, gamma, kT, dt, steps, n = 1.0, 3.0, 3.0, 0.25, 1e-4, 1000, 200000
    rng = np.random.default_rng(41)
    X = np.ones((n, 1))
    P = rng.standard_normal((n, 1)) * math.sqrt(kT * mass)
    P0 = P.copy()
    force = lambda x: -alpha * x
    F = force(X)
    for _ in range(steps):
        X, P, F = O.nvt_langevin_step(force, X, P, F, mass, dt, kT, gamma, None,
                                      rng.standard_normal((n, 1)))
    d = math.sqrt(gamma ** 2 / 4 - alpha / mass)
    b1, b2 = gamma / 2 + d, gamma / 2 - d
    A, B = -b2 / (b1 - b2), b1 / (b1 - b2)
    Z = kT / (2 * d * mass)
    t = steps * dt
    pos = A * math.exp(-b1 * t) + B * math.exp(-b2 * t)
    mom = Z * (-b2 * math.exp(-b2 * t) + b1 * math.exp(-b1 * t)) * mass ** 2
    se_x = X.std() / math.sqrt(n)
    pp = P * P0
    se_p = pp.std() / math.sqrt(n)
    assert abs(X.mean() - pos) <= 4 * se_x + 1e-3 * abs(pos), (X.mean(), pos, se_x)
    assert abs(pp.mean() - mom) <= 4 * se_p + 1e-3 * abs(mom), (pp.mean(), mom, se_p)
    # and the bound is not met trivially: the start is more than 4 SE from the theory
    assert abs(1.0 - pos) > 4 * se_x and abs(kT * mass - mom) > 4 * se_p


def test_langevin_equilibrium_temperature():
    """tests/simulate_test.py:827-870: particles in harmonic wells with masses
    U[0.1, 10] thermalise to the bath: the mean kinetic temperature of the
    later half of the run is within 0.1 of kT."""
    rng = np.random.default_rng(43)
    n, dim, dt, gamma = 2000, 3, 1e-2, 0.3
    R0 = rng.standard_normal((n, dim))
    R = rng.standard_normal((n, dim))
    mass = rng.uniform(0.1, 10.0, n)
    kT = float(rng.uniform(0.3, 1.4))
    force = lambda x: -2.0 * (x - R0)
    P = rng.standard_normal((n, dim)) * np.sqrt(mass)[:, None]
    F = force(R)
    Ts = []
    for step in range(6000):
        R, P, F = O.nvt_langevin_step(force, R, P, F, mass, dt, kT, gamma, None,
                                      rng.standard_normal((n, dim)))
        if step > 3000 and step % 100 == 0:
            Ts.append(float((P * P / mass[:, None]).sum() / (n * dim)))
    assert abs(np.mean(Ts) - kT) < 0.1, (np.mean(Ts), kT)


@pytest.mark.parametrize('dim', [2, 3])
def test_oracle_dense_rows_of_a_subset_match_build(dim):
    """NeighborListOracle.dense_rows (the rows of chosen atoms, for systems too
    large for build's candidate array) equals build's rows, order included."""
    box = np.array([9.0, 7.5] if dim == 2 else [9.0, 6.0, 7.25], np.float32)
    R = random_box(700, dim, box, seed=5)
    onl = O.NeighborListOracle(box, np.float32(1.0), np.float32(0.2))
    full = onl.allocate(R)
    atoms = np.arange(0, 700, 13)
    rows, counts = onl.dense_rows(R, atoms, full.cell_list_capacity)
    w = full.idx.shape[1]
    assert np.array_equal(rows[:, :w], full.idx[atoms])
    assert np.all(rows[:, w:] == 700)
    assert np.array_equal(counts, (full.idx[atoms] < 700).sum(1))


def _jammed_npt_system():
    g = np.load(GOLDEN / 'jammed_soft_sphere_2d.npz')
    spec = O.PairSpec(kind='soft_sphere', sigma=g['sigma'], epsilon=1.0, alpha=2.0,
                      species=g['species'])

    def force_stress(R, box):
        E, F, W = O.all_pairs_energy_forces(spec, R, O.PeriodicGeneral(box))
        return E, F, float(np.trace(W))
    return g, spec, force_stress


def test_npt_nose_hoover_jammed_conserves_invariant():
    """tests/simulate_test.py:360-400 on the oracle: NPT Nose-Hoover of the
    golden jammed soft-sphere packing in its periodic_general cell (kT 1e-3,
    dt 1e-3, target pressure the packing's own) keeps the extended
    Hamiltonian to the reference's f64 tolerance (1.2e-4) over 800 steps and
    the pressure near its target (5%)."""
    g, spec, fs = _jammed_npt_system()
    R = g['fractional_position']
    kT, dt, Pt = 1e-3, 1e-3, float(g['pressure'])
    P = O.maxwell_boltzmann(len(R), 2, kT, seed=3, dtype=np.float64)
    s = O.npt_init(fs, R, P, g['box'], 1.0, kT, dt)
    H0 = O.npt_invariant(fs(s['R'], O.npt_box(s)[0])[0], s, Pt, kT)
    for _ in range(800):
        s = O.npt_nose_hoover_step(fs, s, Pt, kT, dt)
        box, V = O.npt_box(s)
        E, _, dUdV = fs(s['R'], box)
        H = O.npt_invariant(E, s, Pt, kT)
        assert abs(H - H0) <= 1.2e-4 * max(1.0, abs(H0)), (H, H0)
        p = (2 * O.kinetic_energy(s['P']) - dUdV) / (2 * V)
        assert abs(p - Pt) <= 0.05 + 0.05 * abs(Pt), (p, Pt)
