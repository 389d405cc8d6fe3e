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


def test_compute_without_gpu_fails_loudly():
    import torch
    if torch.cuda.is_available():
        pytest.skip('a GPU is present')
    from jax_md_gb300 import partition, space, _native
    disp, _ = space.periodic(10.0)
    fns = partition.neighbor_list(disp, 10.0, 1.0, 0.1)
    with pytest.raises(_native.NativeError):
        fns.allocate(torch.zeros((4, 3)))
