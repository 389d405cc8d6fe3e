"""space.periodic_general, transform and inverse (space.py:109-185, 332-468)
on CPU tensors against the oracle's pinned PeriodicGeneral, the reference's
gradient semantics for fractional coordinates, and the kernels' refusal of
general cells."""
import numpy as np
import pytest
import torch

from jax_md_gb300 import energy, partition, space
from oracle import md_oracle as O


def _cell(dim, seed):
    rng = np.random.default_rng(seed)
    T = np.triu(rng.uniform(-0.6, 0.6, (dim, dim))) + np.diag(rng.uniform(4.0, 6.0, dim))
    return T, rng


@pytest.mark.parametrize('fractional', [True, False])
@pytest.mark.parametrize('dim', [2, 3])
def test_periodic_general_matches_oracle(dim, fractional):
    T, rng = _cell(dim, 10 + dim)
    U = rng.uniform(0.0, 1.0, (40, dim))
    R = U if fractional else U @ T.T
    dR = rng.standard_normal((40, dim))
    disp, shift = space.periodic_general(torch.tensor(T), fractional_coordinates=fractional)
    ref = O.PeriodicGeneral(T, fractional_coordinates=fractional)
    Rt = torch.tensor(R)
    got = disp(Rt[:, None], Rt[None]).numpy()
    np.testing.assert_allclose(got, ref.displacement(R[:, None], R[None]), atol=1e-12)
    np.testing.assert_allclose(shift(Rt, torch.tensor(dR)).numpy(), ref.shift(R, dR), atol=1e-12)
    T2 = T * 0.9
    for kw in ({'box': T2}, {'new_box': T2}):
        got = disp(Rt[:, None], Rt[None], **{k: torch.tensor(v) for k, v in kw.items()}).numpy()
        np.testing.assert_allclose(got, ref.displacement(R[:, None], R[None], **kw), atol=1e-12)
        got = shift(Rt, torch.tensor(dR), **{k: torch.tensor(v) for k, v in kw.items()}).numpy()
        np.testing.assert_allclose(got, ref.shift(R, dR, **kw), atol=1e-12)


def test_periodic_general_unwrapped_and_perturbation():
    T, rng = _cell(3, 4)
    U = rng.uniform(0.0, 1.0, (20, 3))
    dR = 3.0 * rng.standard_normal((20, 3))
    _, sh = space.periodic_general(T, wrapped=False)
    np.testing.assert_allclose(sh(torch.tensor(U), torch.tensor(dR)).numpy(),
                               O.PeriodicGeneral(T, wrapped=False).shift(U, dR), atol=1e-12)
    disp, _ = space.periodic_general(T)
    eps = np.eye(3) + 0.01 * rng.standard_normal((3, 3))
    Ut = torch.tensor(U)
    got = disp(Ut[:, None], Ut[None], perturbation=torch.tensor(eps)).numpy()
    want = np.einsum('ij,...j->...i', eps, O.PeriodicGeneral(T).displacement(U[:, None], U[None]))
    np.testing.assert_allclose(got, want, atol=1e-12)


def test_transform_inverse_roundtrip_and_pass_through_derivative():
    """space_test.py:88-170: transform(inverse(T), transform(T, R)) = R, and
    the derivative in R passes through unchanged (space.py:155-185)."""
    T, rng = _cell(3, 6)
    R = torch.tensor(rng.standard_normal((7, 3)), requires_grad=True)
    X = space.transform(torch.tensor(T), R)
    np.testing.assert_allclose(space.transform(space.inverse(torch.tensor(T)), X).detach().numpy(),
                               R.detach().numpy(), atol=1e-12)
    g = torch.tensor(rng.standard_normal((7, 3)))
    (X * g).sum().backward()
    np.testing.assert_array_equal(R.grad.numpy(), g.numpy())
    for box in (2.5, np.array([2.0, 3.0, 4.0])):
        np.testing.assert_allclose(space.transform(box, R.detach()).numpy(),
                                   O.transform(box, R.detach().numpy()), atol=1e-14)


@pytest.mark.parametrize('dim', [2, 3])
def test_fractional_gradients_are_real_space(dim):
    """space_test.py:351-400, 530-549: the gradient of an energy of
    fractional positions equals the real-space gradient of the same energy
    in real coordinates (diagonal and triclinic cells)."""
    T, rng = _cell(dim, 20 + dim)
    U = rng.uniform(0.0, 1.0, (30, dim))

    def energy_of(disp, R):
        d = disp(R[:, None], R[None])
        r2 = (d * d).sum(-1) + torch.eye(len(R), dtype=R.dtype)
        return (1.0 / r2).sum()
    for cell in (np.diag(np.diag(T)), T):
        df, _ = space.periodic_general(torch.tensor(cell))
        dr, _ = space.periodic_general(torch.tensor(cell), fractional_coordinates=False)
        Uf = torch.tensor(U, requires_grad=True)
        Rr = torch.tensor(U @ cell.T, requires_grad=True)
        energy_of(df, Uf).backward()
        energy_of(dr, Rr).backward()
        np.testing.assert_allclose(Uf.grad.numpy(), Rr.grad.numpy(), rtol=1e-9, atol=1e-9)
    # the diagonal cell in real coordinates is space.periodic
    side = np.diag(T)
    dp, _ = space.periodic(side.tolist())
    Rp = torch.tensor(U * side, requires_grad=True)
    energy_of(dp, Rp).backward()
    dr, _ = space.periodic_general(torch.tensor(np.diag(side)), fractional_coordinates=False)
    Rr = torch.tensor(U * side, requires_grad=True)
    energy_of(dr, Rr).backward()
    np.testing.assert_allclose(Rp.grad.numpy(), Rr.grad.numpy(), rtol=1e-9, atol=1e-9)


def test_general_cell_geometry_for_the_kernels():
    """periodic_general with fractional coordinates becomes the kernels'
    general-cell geometry (unit-cube minimum image, T and T^-1); cells the
    kernels cannot take are refused on the host."""
    from jax_md_gb300 import _native as N
    T = np.array([[8.0, 1.5, -0.5], [0.0, 7.0, 2.0], [0.0, 0.0, 9.0]])
    disp, shift = space.periodic_general(T)
    s = disp.space(3)
    assert s.periodic == N.GENERAL_CELL and list(s.box) == [1.0, 1.0, 1.0]
    np.testing.assert_allclose(np.array(s.cell).reshape(3, 3), T, rtol=1e-7)
    np.testing.assert_allclose(np.array(s.inv_cell).reshape(3, 3), np.linalg.inv(T), rtol=1e-6)
    assert shift.space(3).periodic == N.GENERAL_CELL
    # the box keyword replaces the cell
    np.testing.assert_allclose(np.array(disp.space(3, box=2 * T).cell).reshape(3, 3), 2 * T,
                               rtol=1e-7)
    # 2D cells sit in the upper-left block
    s2 = space.periodic_general(np.array([[5.0, 1.0], [0.0, 4.0]]))[0].space(2)
    assert list(s2.cell) == [5.0, 1.0, 0.0, 0.0, 4.0, 0.0, 0.0, 0.0, 1.0]
    with pytest.raises(ValueError, match='upper-triangular'):
        space.periodic_general(T.T)[0].space(3)
    # real coordinates: an orthorhombic cell is space.periodic, a skewed one is refused
    d_real, _ = space.periodic_general(np.diag([5.0, 6.0, 7.0]), fractional_coordinates=False)
    sr = d_real.space(3)
    assert sr.periodic == 1 and list(sr.box) == [5.0, 6.0, 7.0]
    with pytest.raises(NotImplementedError, match='fractional'):
        space.periodic_general(T, fractional_coordinates=False)[0].space(3)
    # the orthorhombic displacement refuses a box keyword, as space.periodic does
    with pytest.raises(space.UnexpectedBoxException):
        space.periodic(5.0)[0].space(3, box=T)


def _triclinic(rng, L):
    """An upper-triangular cell from edge lengths in [L/2, 3L] and angles in
    [45, 125] degrees, the construction of the reference's general-cell tests
    (tests/partition_test.py:536-560); None when the angles admit no cell."""
    a, b, c = rng.uniform(0.5 * L, 3 * L, 3)
    al, be, ga = np.radians(rng.uniform(45.0, 125.0, 3))
    xx, yy, xy, xz = a, b * np.sin(ga), b * np.cos(ga), c * np.cos(be)
    yz = (b * c * np.cos(al) - xy * xz) / yy
    zz2 = c * c - xz * xz - yz * yz
    if zz2 <= 0:
        return None
    return np.array([[xx, xy, xz], [0.0, yy, yz], [0.0, 0.0, np.sqrt(zz2)]])


def test_fractional_cell_size_matches_oracle_and_geometry():
    """partition.fractional_cell_size (partition.py:595-634) agrees with the
    oracle's restatement, and 1 / cell size cells per side never exceed the
    perpendicular widths V / |b x c|, V / |c x a|, V / |a x b| over the cutoff."""
    rng = np.random.default_rng(11)
    done = 0
    while done < 20:
        T = _triclinic(rng, 12.0)
        if T is None:
            continue
        done += 1
        for cut in (1.0, 2.5, 3.3):
            got = partition.fractional_cell_size(T, cut)
            assert got == O.fractional_cell_size(T, cut)
            a, b, c = T[:, 0], T[:, 1], T[:, 2]
            V = abs(np.linalg.det(T))
            widths = [V / np.linalg.norm(np.cross(b, c)), V / np.linalg.norm(np.cross(c, a)),
                      V / np.linalg.norm(np.cross(a, b))]
            n = round(1.0 / float(got))
            assert n == max(1, int(np.floor(min(widths) / cut)))
    for box, cut in ((3.0, 0.11), (np.array([4.0, 5.0, 6.0]), 1.2),
                     (np.array([[5.0, 1.0], [0.0, 4.0]]), 1.1)):
        assert partition.fractional_cell_size(box, cut) == O.fractional_cell_size(box, cut)


def test_oracle_fractional_cell_list_equals_all_pairs():
    """The oracle's fractional cell list finds the pairs its all-pairs search
    finds in random triclinic cells (the reference's test_general_unit_cell
    and test_issue191_1, partition_test.py:462-563)."""
    rng = np.random.default_rng(12)
    L = (128 / 0.05) ** (1 / 3)
    done = 0
    while done < 6:
        T = _triclinic(rng, L)
        if T is None:
            continue
        T = T.astype(np.float32).astype(np.float64)
        U = rng.uniform(0, 1, (128, 3)).astype(np.float32)
        sp = O.PeriodicGeneral(T)
        with_cells = O.NeighborListOracle(T, 2.5, capacity_multiplier=1.0, space=sp,
                                          fractional=True)
        if not (with_cells.bin_min < 1 / 3):
            continue
        done += 1
        allp = O.NeighborListOracle(T, 2.5, disable_cell_list=True, space=sp, fractional=True)
        a = with_cells.allocate(U)
        b = allp.allocate(U)
        assert a.use_cell_list and not b.use_cell_list
        np.testing.assert_array_equal(np.sort(a.idx, -1)[:, :a.max_occupancy],
                                      np.sort(b.idx, -1)[:, :a.max_occupancy])


def test_map_product_layout():
    """space.py:480-484: out[b, a] = displacement(Ra[a], Rb[b]), for periodic
    and periodic_general displacements and for metrics."""
    rng = np.random.default_rng(3)
    Ra, Rb = rng.uniform(0, 5, (6, 3)), rng.uniform(0, 5, (4, 3))
    d, _ = space.periodic(5.0)
    got = space.map_product(d)(torch.tensor(Ra), torch.tensor(Rb)).numpy()
    assert got.shape == (4, 6, 3)
    for b in range(4):
        for a in range(6):
            np.testing.assert_allclose(got[b, a], O.displacement(Ra[a], Rb[b], np.full(3, 5.0)),
                                       atol=1e-12)
    T = np.array([[5.0, 0.4, 0.0], [0.0, 5.0, 0.3], [0.0, 0.0, 5.0]])
    dg, _ = space.periodic_general(T)
    Ua, Ub = Ra / 5.0, Rb / 5.0
    got = space.map_product(dg)(torch.tensor(Ua), torch.tensor(Ub)).numpy()
    np.testing.assert_allclose(got[2, 5], O.PeriodicGeneral(T).displacement(Ua[5], Ub[2]), atol=1e-12)
    m = space.map_product(space.metric(d))(torch.tensor(Ra), torch.tensor(Rb)).numpy()
    np.testing.assert_allclose(m[1, 3], np.linalg.norm(O.displacement(Ra[3], Rb[1], np.full(3, 5.0))),
                               atol=1e-12)


def test_integrator_geometry_of_general_shifts():
    """A wrapped fractional shift of periodic_general drives the integrator
    kernels with the general-cell geometry (u <- mod(u + T^-1 dR, 1));
    an unwrapped fractional shift is refused."""
    from jax_md_gb300 import _native as N, simulate
    _, shift = space.periodic_general(np.eye(3) * 8.0)
    assert simulate._shift_space(shift, 3).periodic == N.GENERAL_CELL
    _, shift_u = space.periodic_general(np.eye(3) * 8.0, wrapped=False)
    with pytest.raises(NotImplementedError, match='wrapped'):
        simulate._shift_space(shift_u, 3)
