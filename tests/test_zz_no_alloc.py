"""jmd_kinetic_energy_static_scratch (no allocation) against jmd_kinetic_energy.

The static-scratch entry point shares one device array across calls; this
file is collected last so that it also runs after every other test has used
the library, and it must pass alone in a fresh process too.
"""
import pytest
import torch

from jax_md_gb300 import _native as N


def _ke_workspace(L, p, mass, m0, n, dim, cuda):
    ws = torch.empty(L.jmd_reduce_workspace_bytes(n), dtype=torch.uint8, device=cuda)
    out = torch.empty((), dtype=torch.float64, device=cuda)
    N.check(L.jmd_kinetic_energy(p.data_ptr(), p.stride(0), N.ptr(mass), m0, n, dim,
                                 out.data_ptr(), ws.data_ptr(), ws.numel(), N.stream_ptr()),
            'kinetic_energy')
    return out


@pytest.mark.gpu
@pytest.mark.parametrize('n,dim,per_atom_mass', [(864000, 3, False), (100003, 3, True),
                                                 (4097, 2, False), (1, 3, False)])
def test_static_scratch_matches_workspace_path(cuda, n, dim, per_atom_mass):
    L = N.lib()
    gen = torch.Generator(device=cuda).manual_seed(n)
    p = torch.randn((n, 4), generator=gen, device=cuda)
    mass = (torch.rand(n, generator=gen, device=cuda) + 0.5) if per_atom_mass else None
    m0 = 1.7
    ref = _ke_workspace(L, p, mass, m0, n, dim, cuda)
    outs = []
    for _ in range(2):  # two calls in a row reuse the shared array
        o = torch.empty((), dtype=torch.float64, device=cuda)
        N.check(L.jmd_kinetic_energy_static_scratch(p.data_ptr(), 4, N.ptr(mass), m0, n, dim,
                                                    o.data_ptr(), N.stream_ptr()),
                'kinetic_energy_static_scratch')
        outs.append(o)
    torch.cuda.synchronize()
    r = float(ref)
    for o in outs:
        assert abs(float(o) - r) <= 1e-12 * abs(r), (float(o), r)


def test_static_scratch_rejects_oversized_systems():
    """The size check runs on the host before any CUDA call."""
    import ctypes
    L = N.lib()
    out = ctypes.c_double(0.0)  # never written: the call returns before any CUDA call
    rc = L.jmd_kinetic_energy_static_scratch(None, 4, None, 1.0, 4194305, 3,
                                             ctypes.addressof(out), None)
    assert rc == 1
    assert b'4194304' in L.jmd_last_error()
