"""The C-ABI library builds, loads, and exports every symbol its header declares.

CPU only: no kernel is launched (there is no GPU here); the product path must
fail loudly without one.
"""
import ctypes
import re
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
HEADERS = sorted((ROOT / 'include').glob('*.h'))


def declared_symbols():
    names = set()
    for h in HEADERS:
        text = re.sub(r'/\*.*?\*/', '', h.read_text(), flags=re.S)
        for m in re.finditer(r'\b(jmd_[a-z0-9_]+)\s*\(', text):
            names.add(m.group(1))
    return sorted(names)


@pytest.fixture(scope='module')
def lib():
    from jax_md_gb300 import _build
    path = _build.build()
    return ctypes.CDLL(str(path))


def test_header_declares_entry_points():
    names = declared_symbols()
    for must in ('jmd_neighbor_list_build', 'jmd_pair_forces', 'jmd_verlet_kick_drift',
                 'jmd_nhc_half_step', 'jmd_skin_check', 'jmd_cell_list_build'):
        assert must in names


def test_library_exports_every_declared_symbol(lib):
    missing = [n for n in declared_symbols() if not hasattr(lib, n)]
    assert not missing, missing


def test_python_binding_covers_header():
    from jax_md_gb300 import _native
    bound = set(_native.SIGNATURES)
    missing = [n for n in declared_symbols() if n not in bound]
    assert not missing, missing


def test_host_only_queries(lib):
    from jax_md_gb300 import _native as N
    L = N.lib()
    assert L.jmd_version() == 1
    nl = N.NList()
    nl.space.dim = 3
    nl.space.periodic = 1
    nl.use_cell_list = 1
    for d in range(3):
        nl.cells_per_side[d] = 35
        nl.cell_size[d] = 2.88
        nl.space.box[d] = 100.0
    nl.cell_capacity = 40
    assert L.jmd_neighbor_list_workspace_bytes(ctypes.byref(nl), 864000) > 864000 * 16
    assert L.jmd_pair_workspace_bytes(864000) > 0


def test_invalid_arguments_are_reported(lib):
    from jax_md_gb300 import _native as N
    L = N.lib()
    nl = N.NList()
    nl.space.dim = 5
    rc = L.jmd_neighbor_list_build(ctypes.byref(nl), None, 4, 0, None, 0, None, None, None, None,
                                   0, None, None, 0, None)
    assert rc != 0
    assert b'dim' in L.jmd_last_error()


def test_batched_nose_hoover_arguments_are_checked(lib):
    """The batched chain entries reject bad arguments before any launch."""
    import numpy as np
    from jax_md_gb300 import _native as N
    L = N.lib()
    assert L.jmd_batch_nvt_run(None, None, 1, 0, None) != 0
    dummy = np.zeros(16, np.int64)
    b = N.Batch()
    b.dim, b.n_systems, b.n_atoms, b.total_cells, b.max_cells = 3, 1, 4, 1, 1
    for f in ('sys_offset', 'atom_sys', 'box', 'cell_offset', 'cells_per_side', 'cell_size'):
        setattr(b, f, dummy.ctypes.data)
    c = N.Nhc()
    c.chain_length, c.chain_steps, c.sy_steps, c.dt, c.tau = 9, 2, 3, 0.005, 0.5
    ptr = dummy.ctypes.data
    rc = L.jmd_batch_nhc_half_step_vjp(ctypes.byref(b), ctypes.byref(c), ptr, ptr, 1, ptr, ptr,
                                       ptr, ptr, None)
    assert rc != 0 and b'chain_length 2..7' in L.jmd_last_error()
    v = N.BatchNvt()
    v.chain = c
    v.chain.chain_length, v.chain.sy_steps = 5, 4
    v.chain_state = ptr
    rc = L.jmd_batch_nhc_half_step(ctypes.byref(b), ctypes.byref(v), None, None, 1.0, 1, 0, None,
                                   None, None)
    assert rc != 0 and b'sy_steps' in L.jmd_last_error()
    b.dim = 4
    rc = L.jmd_batch_nhc_half_step(ctypes.byref(b), ctypes.byref(v), None, None, 1.0, 1, 0, None,
                                   None, None)
    assert rc != 0 and b'dim' in L.jmd_last_error()


def test_compute_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    from jax_md_gb300 import partition, space, _native
    disp, _ = space.periodic(10.0)
    fns = partition.neighbor_list(disp, 10.0, 1.0, 0.1)
    with pytest.raises(_native.NativeError):
        fns.allocate(torch.zeros((4, 3)))
