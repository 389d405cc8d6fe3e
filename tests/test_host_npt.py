"""Host pieces of simulate.npt_nose_hoover (no device needed): the sinh(x)/x
series, the box of a state, and the refusals of the integrator."""
import math

import numpy as np
import pytest
import torch


def test_sinhx_x_matches_sinh_over_x():
    """simulate.py:763-772: the Taylor series of sinh(x)/x through x^10; it
    differs from sinh(x)/x by about the first omitted term, x^12 / 13!."""
    from jax_md_gb300 import simulate
    assert simulate.sinhx_x(0.0) == 1.0
    for x in (1e-6, 1e-3, 0.05, 0.3, 1.0):
        err = abs(simulate.sinhx_x(x) - math.sinh(x) / x)
        assert err <= 1e-15 + 1.1 * x ** 12 / math.factorial(13), (x, err)


def test_npt_box_follows_box_position():
    """simulate.py:775-792: V = V_0 exp(d box_position), box = (V / V_0)^(1/d) T."""
    from jax_md_gb300 import simulate
    T = np.array([[5.0, 1.0, 0.5], [0.0, 6.0, -0.25], [0.0, 0.0, 7.0]])
    st = simulate.NPTNoseHooverState(torch.zeros((4, 3)), torch.zeros((4, 3)), torch.zeros((4, 3)),
                                     1.0, T, 0.01, 0.0, 1.0, 0.0, None, None)
    V, box_fn = simulate._npt_box_info(st)
    assert abs(V - np.linalg.det(T) * math.exp(3 * 0.01)) < 1e-9 * V
    np.testing.assert_allclose(simulate.npt_box(st), math.exp(0.01) * T, rtol=1e-12)
    np.testing.assert_allclose(box_fn(np.linalg.det(T)), T, rtol=1e-12)


def test_npt_needs_a_general_shift():
    from jax_md_gb300 import energy, simulate, space
    disp, shift = space.periodic(10.0)
    _, efn = energy.lennard_jones_neighbor_list(disp, 10.0)
    with pytest.raises(NotImplementedError, match='periodic_general'):
        simulate.npt_nose_hoover(efn, shift, 1e-3, 1.0, 1.0)
