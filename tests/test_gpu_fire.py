"""FIRE minimisation on the GPU against the FP64 oracle (minimize.py:124-226)."""
import numpy as np
import pytest
import torch

from oracle import md_oracle as O

pytestmark = pytest.mark.gpu


def _ss_system(cuda, n=600, seed=3):
    from jax_md_gb300 import energy, partition, space
    R, L, species = O.bidisperse_2d(n, phi=0.84, seed=seed)
    sigma = np.array([[1.0, 1.2], [1.2, 1.4]])
    disp, shift = space.periodic(float(L))
    nfn, efn = energy.soft_sphere_neighbor_list(disp, float(L), torch.tensor(species, device=cuda),
                                                sigma=sigma, format=partition.Dense)
    return R, float(L), species, sigma, shift, nfn, efn


def test_fire_matches_oracle_steps(cuda):
    from jax_md_gb300 import minimize
    R, L, species, sigma, shift, nfn, efn = _ss_system(cuda)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    init, apply = minimize.fire_descent(efn, shift)
    st = init(Rt, neighbor=nb)
    spec = O.PairSpec(kind='soft_sphere', sigma=sigma, species=species)
    box = np.full(2, L)
    nl = O.NeighborListOracle(box, 1.4, 0.2, fmt=O.DENSE)
    h = {'nb': nl.allocate(R)}

    def fn(X):
        h['nb'] = nl.update(X, h['nb'])
        return O.pair_energy_forces(spec, X, h['nb'].idx, O.DENSE, box)[1]
    Rd = R.astype(np.float64)
    s = O.FireO(Rd, np.zeros_like(Rd), fn(Rd), 1.0, 0.1, 0.1, 0)
    for k in range(25):
        nb = nb.update(st.position)
        st = apply(st, neighbor=nb)
        s = O.fire_step(fn, s, box)
    torch.cuda.synchronize()
    assert abs(float(st.dt) - s.dt) < 1e-5 * max(1.0, s.dt)
    assert abs(float(st.alpha) - s.alpha) < 1e-5
    assert int(st.n_pos) == s.n_pos
    d = O.displacement(st.position.contiguous().cpu().numpy(), s.R, box)
    assert np.abs(d).max() < 1e-3


def test_fire_minimises(cuda):
    from jax_md_gb300 import minimize
    R, L, species, sigma, shift, nfn, efn = _ss_system(cuda, n=1000, seed=5)
    Rt = torch.tensor(R, device=cuda)
    nb = nfn.allocate(Rt)
    init, apply = minimize.fire_descent(efn, shift)
    st = init(Rt, neighbor=nb)
    E0 = float(efn.energy_f64(st.position, nb))
    for _ in range(2000):
        nb = nb.update(st.position)
        st = apply(st, neighbor=nb)
    assert not bool(nb.did_buffer_overflow)
    E1 = float(efn.energy_f64(st.position, nb))
    fmax = float(st.force.abs().max())
    assert E1 < 0.2 * E0
    assert fmax < 1e-2
