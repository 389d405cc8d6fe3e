"""jax_md.util's numerical helpers and simulate.canonicalize_momenta on CPU
tensors (util.py:85-112, simulate.py:162-165)."""
import numpy as np
import torch

from jax_md_gb300 import simulate, util


def test_high_precision_sum_accumulates_in_f64():
    x = torch.full((1 << 22,), 0.1, dtype=torch.float32)
    s = util.high_precision_sum(x)
    assert s.dtype == torch.float32
    assert float(s) == float(np.float32(np.float64(np.float32(0.1)) * (1 << 22)))
    m = torch.arange(12, dtype=torch.float32).reshape(3, 4)
    torch.testing.assert_close(util.high_precision_sum(m, axis=1), m.sum(1))
    assert util.high_precision_sum(m, axis=(0, 1), keepdims=True).shape == (1, 1)
    assert util.high_precision_sum(m, keepdims=True).shape == (1, 1)
    i = torch.tensor([2 ** 30, 2 ** 30], dtype=torch.int32)
    assert util.high_precision_sum(i).dtype == torch.int32


def test_safe_mask_and_downcast():
    r2 = torch.tensor([0.0, 4.0, 9.0], requires_grad=True)
    d = util.safe_mask(r2 > 0, torch.sqrt, r2, placeholder=-1.0)
    assert d.tolist() == [-1.0, 2.0, 3.0]
    assert util.maybe_downcast(1.5).dtype == torch.float32
    t = torch.ones(2, dtype=torch.float64)
    assert util.maybe_downcast(t) is t
    assert util.maybe_downcast(np.ones(2)).dtype == torch.float32


def test_canonicalize_momenta():
    st = simulate.NVEState(torch.zeros((3, 2)), torch.zeros((3, 2)), torch.zeros((3, 2)), 1.0)
    assert simulate.canonicalize_momenta(st, None) is st
    p = torch.arange(6, dtype=torch.float32).reshape(3, 2)
    new = simulate.canonicalize_momenta(st, p)
    assert torch.equal(new.momentum, p) and new.momentum.stride(0) == 4


def test_dispatch_by_state_registry():
    """simulate.py:100-116: step functions dispatch on the type of
    state.position; registered implementations replace the default one for
    their type only."""
    class Rigid:
        pass

    class State:
        def __init__(self, pos):
            self.position = pos
    seen = []
    for step in (simulate.momentum_step, simulate.position_step, simulate.stochastic_step):
        step.register(Rigid)(lambda state, *a, _n=step.__name__, **k: seen.append(_n) or state)
    st = State(Rigid())
    simulate.momentum_step(st, 0.1)
    simulate.position_step(st, None, 0.1)
    simulate.stochastic_step(st, 0.1, 1.0, 0.5)
    assert seen == ['momentum_step', 'position_step', 'stochastic_step']
    for step in (simulate.momentum_step, simulate.position_step, simulate.stochastic_step):
        step._registry.pop(Rigid)
    simulate.kinetic_energy.register(Rigid)(lambda state: 1.25)
    simulate.temperature.register(Rigid)(lambda state: 0.5)
    assert simulate.kinetic_energy(st) == 1.25 and simulate.temperature(st) == 0.5
    simulate.kinetic_energy._registry.pop(Rigid)
    simulate.temperature._registry.pop(Rigid)


def test_gradient_descent_on_a_harmonic_well():
    """minimize.py:65-94 with a Python energy: each step moves R by
    step_size F(R), so a harmonic well contracts by (1 - step_size k)."""
    from jax_md_gb300 import minimize, space
    _, shift = space.free()
    k, step = 2.0, 0.1
    init, apply = minimize.gradient_descent(lambda R, **kw: 0.5 * k * (R * R).sum(), shift, step)
    R = init(torch.tensor([[1.0, -2.0], [0.5, 0.25]], dtype=torch.float64))
    for _ in range(5):
        R = apply(R)
    np.testing.assert_allclose(R.detach().numpy(),
                               np.array([[1.0, -2.0], [0.5, 0.25]]) * (1 - step * k) ** 5,
                               rtol=1e-12)


def test_setup_quantities_and_clipped_force():
    """quantity.py:592-660 (unit-ball volume, particle volume, volume
    fraction, box sizes), quantity.py:63-73 (clipped force) and
    partition.py:676-681 (box validity)."""
    import math
    from jax_md_gb300 import partition, quantity
    assert math.isclose(quantity.nball_unit_volume(2), math.pi)
    assert math.isclose(quantity.nball_unit_volume(3), 4 * math.pi / 3)
    # the 2D bidisperse packing of the batched workload: phi = 0.84
    radii = np.array([0.5, 0.7])
    species = np.array([0, 1, 1, 0, 1, 0])
    L = quantity.box_size_at_volume_fraction(0.84, radii, 2, species=species)
    assert math.isclose(quantity.volume_fraction(L, radii, 2, species=species), 0.84)
    assert math.isclose(L, math.sqrt(3 * math.pi * (0.25 + 0.49) / 0.84))
    assert math.isclose(quantity.box_size_at_number_density(864000, 0.8442, 3),
                        (864000 / 0.8442) ** (1 / 3))
    f = quantity.clipped_force(lambda R: 0.5 * 100.0 * (R * R).sum(), 1.0)
    F = f(torch.tensor([[0.001, 0.0], [3.0, 4.0]], dtype=torch.float64))
    np.testing.assert_allclose(F.numpy(), [[-0.1, 0.0], [-0.6, -0.8]], rtol=1e-12)
    assert partition.is_box_valid(5.0) and partition.is_box_valid(np.ones(3))
    assert partition.is_box_valid(np.triu(np.ones((3, 3))))
    assert not partition.is_box_valid(np.ones((3, 3)))
