"""ctypes binding of the C ABI in ``include/jax_md_gb300.h``.

The shared library is the only compute path: if it is missing or no CUDA
device is present, every call raises.  PyTorch supplies device memory and the
current CUDA stream; the library sees only raw pointers.
"""
from __future__ import annotations

import ctypes as C
import os
from pathlib import Path

import torch

PKG = Path(__file__).resolve().parent
LIB_PATH = PKG / 'libjaxmd_gb300.so'

MAX_SPECIES = 8
DENSE, SPARSE, ORDERED_SPARSE = 0, 1, 2
LJ, LJ_TRUNCATED, SOFT_SPHERE, MORSE = 0, 1, 2, 3

NEIGHBOR_LIST_OVERFLOW = 1
CELL_LIST_OVERFLOW = 2
CELL_SIZE_TOO_SMALL = 4
MALFORMED_BOX = 8


GENERAL_CELL = 2  # jmd_space.periodic of a general cell (JMD_GENERAL_CELL)


class Space(C.Structure):
    _fields_ = [('dim', C.c_int32), ('periodic', C.c_int32), ('box', C.c_float * 3),
                ('cell', C.c_float * 9), ('inv_cell', C.c_float * 9)]


class NList(C.Structure):
    _fields_ = [('space', Space), ('cutoff_sq', C.c_float), ('use_cell_list', C.c_int32),
                ('cells_per_side', C.c_int32 * 3), ('cell_size', C.c_float * 3),
                ('cell_capacity', C.c_int32), ('format', C.c_int32), ('mask_self', C.c_int32),
                ('max_occupancy', C.c_int64)]


class Pair(C.Structure):
    _fields_ = [('kind', C.c_int32), ('n_species', C.c_int32), ('per_pair_cutoff', C.c_int32),
                ('pad_', C.c_int32), ('r_onset', C.c_float), ('r_cutoff', C.c_float),
                ('sigma', (C.c_float * MAX_SPECIES) * MAX_SPECIES),
                ('epsilon', (C.c_float * MAX_SPECIES) * MAX_SPECIES),
                ('alpha', (C.c_float * MAX_SPECIES) * MAX_SPECIES),
                ('particle_sigma', C.c_void_p), ('particle_epsilon', C.c_void_p)]


class Nhc(C.Structure):
    _fields_ = [('chain_length', C.c_int32), ('chain_steps', C.c_int32), ('sy_steps', C.c_int32),
                ('dof', C.c_int32), ('dt', C.c_double), ('tau', C.c_double)]


class NveSystem(C.Structure):
    _fields_ = [('n', C.c_int64), ('space', Space), ('position', C.c_void_p),
                ('position_alt', C.c_void_p), ('momentum', C.c_void_p), ('force', C.c_void_p),
                ('mass', C.c_void_p), ('mass_scalar', C.c_float), ('species', C.c_void_p),
                ('pair', Pair), ('nlist', NList), ('idx', C.c_void_p), ('idx_ld', C.c_int64),
                ('nbr_count', C.c_void_p), ('reference_position', C.c_void_p),
                ('error_code', C.c_void_p), ('occupancy', C.c_void_p),
                ('rebuild_flag', C.c_void_p), ('nl_workspace', C.c_void_p),
                ('nl_workspace_bytes', C.c_size_t), ('dt', C.c_float),
                ('threshold_sq', C.c_float)]


class SortedState(C.Structure):
    _fields_ = [('position_a', C.c_void_p), ('position_b', C.c_void_p), ('momentum', C.c_void_p),
                ('force', C.c_void_p), ('reference_position', C.c_void_p),
                ('scratch4a', C.c_void_p), ('scratch4b', C.c_void_p), ('species', C.c_void_p),
                ('perm', C.c_void_p), ('scratch_i_a', C.c_void_p), ('scratch_i_b', C.c_void_p),
                ('idx', C.c_void_p), ('idx_ld', C.c_int64), ('nbr_count', C.c_void_p),
                ('error_code', C.c_void_p), ('occupancy', C.c_void_p),
                ('rebuild_flag', C.c_void_p), ('workspace', C.c_void_p),
                ('workspace_bytes', C.c_size_t), ('seg_list', C.c_void_p),
                ('seg_list_bytes', C.c_int64), ('seg_cells', C.c_int32), ('seg_threads', C.c_int32),
                ('seg_list_smem', C.c_int32), ('seg_half', C.c_int32), ('flags', C.c_int32),
                ('seg_status', C.c_void_p)]


RUN_SKIP_EXIT_LIST = 1
RUN_WARM_START = 2


class Nvt(C.Structure):
    _fields_ = [('chain', Nhc), ('chain_state', C.c_void_p), ('p_scale', C.c_void_p),
                ('reduce_workspace', C.c_void_p), ('reduce_workspace_bytes', C.c_size_t)]


class Batch(C.Structure):
    _fields_ = [('dim', C.c_int32), ('n_systems', C.c_int32), ('n_atoms', C.c_int64),
                ('total_cells', C.c_int32), ('max_cells', C.c_int32),
                ('sys_offset', C.c_void_p), ('atom_sys', C.c_void_p), ('box', C.c_void_p),
                ('cell_offset', C.c_void_p), ('cells_per_side', C.c_void_p),
                ('cell_size', C.c_void_p)]


class BatchNList(C.Structure):
    _fields_ = [('cutoff_sq', C.c_float), ('max_occupancy', C.c_int32), ('ld', C.c_int32),
                ('mask_self', C.c_int32), ('idx', C.c_void_p), ('count', C.c_void_p),
                ('reference_position', C.c_void_p), ('occupancy', C.c_void_p),
                ('error_code', C.c_void_p), ('rebuild_flag', C.c_void_p),
                ('workspace', C.c_void_p), ('workspace_bytes', C.c_size_t)]


class FireParams(C.Structure):
    _fields_ = [(k, C.c_float) for k in ('dt_start', 'dt_max', 'n_min', 'f_inc', 'f_dec',
                                         'alpha_start', 'f_alpha', 'f_tol')]


class BatchSystem(C.Structure):
    _fields_ = [('batch', Batch), ('nlist', BatchNList), ('pair', Pair), ('species', C.c_void_p),
                ('position', C.c_void_p), ('momentum', C.c_void_p), ('force', C.c_void_p),
                ('mass', C.c_void_p), ('mass_scalar', C.c_float), ('dt', C.c_float),
                ('threshold_sq', C.c_float), ('fire_state', C.c_void_p), ('done', C.c_void_p),
                ('n_done', C.c_void_p)]


class BatchNvt(C.Structure):
    _fields_ = [('chain', Nhc), ('chain_state', C.c_void_p), ('p_scale', C.c_void_p)]


P = C.c_void_p
I64 = C.c_int64
I32 = C.c_int32
F32 = C.c_float
SZ = C.c_size_t

# name -> (restype, argtypes)
SIGNATURES = {
    'jmd_last_error': (C.c_char_p, []),
    'jmd_version': (C.c_int, []),
    'jmd_cell_workspace_bytes': (SZ, [I64, I64]),
    'jmd_cell_max_filling': (C.c_int, [P, I64, I64, C.POINTER(NList), P, P, SZ, P]),
    'jmd_cell_list_build': (C.c_int, [P, I64, I64, C.POINTER(NList), P, P, P, P, P, SZ, P]),
    'jmd_neighbor_list_workspace_bytes': (SZ, [C.POINTER(NList), I64]),
    'jmd_neighbor_list_build': (C.c_int, [C.POINTER(NList), P, I64, I64, P, I64, P, P, P, P, I64,
                                          P, P, SZ, P]),
    'jmd_skin_check': (C.c_int, [P, I64, P, I64, I64, C.POINTER(Space), F32, P, P]),
    'jmd_pair_workspace_bytes': (SZ, [I64]),
    'jmd_set_pair_threads_per_atom': (C.c_int, [C.c_int]),
    'jmd_pair_forces': (C.c_int, [C.POINTER(Pair), C.POINTER(Space), I32, P, I64, P, I64, P, I64,
                                  I64, P, P, I64, P, P, P, P, SZ, P]),
    'jmd_momentum_step': (C.c_int, [P, I64, P, I64, I64, I32, F32, P]),
    'jmd_position_step': (C.c_int, [P, I64, P, I64, P, F32, I64, C.POINTER(Space), F32, P]),
    'jmd_verlet_kick_drift': (C.c_int, [P, I64, P, I64, P, I64, P, F32, I64, C.POINTER(Space), F32,
                                        P, P, I64, F32, P, P]),
    'jmd_reduce_workspace_bytes': (SZ, [I64]),
    'jmd_kinetic_energy': (C.c_int, [P, I64, P, F32, I64, I32, P, P, SZ, P]),
    'jmd_kinetic_energy_static_scratch': (C.c_int, [P, I64, P, F32, I64, I32, P, P]),
    'jmd_nhc_half_step': (C.c_int, [C.POINTER(Nhc), P, P, I32, P, P]),
    'jmd_scale_momentum': (C.c_int, [P, I64, I64, I32, P, P]),
    'jmd_set_dense_threads_per_atom': (C.c_int, [C.c_int]),
    'jmd_set_pair_generic': (C.c_int, [C.c_int]),
    'jmd_nve_fused_step': (C.c_int, [C.POINTER(Pair), C.POINTER(Space), P, P, P, P, F32, P, I64, P,
                                     I64, I64, P, F32, P, F32, P, P]),
    'jmd_force_kick': (C.c_int, [C.POINTER(Pair), C.POINTER(Space), P, P, P, P, I64, P, I64, I64,
                                 P, F32, P]),
    'jmd_nve_run': (C.c_int, [C.POINTER(NveSystem), I64, I32, P]),
    'jmd_engine_clear_cache': (C.c_int, []),
    'jmd_sort_by_cell': (C.c_int, [C.POINTER(NList), P, P, P, P, P, I64, P, P, P, P, P, P, SZ, P]),
    'jmd_nve_run_sorted': (C.c_int, [C.POINTER(NveSystem), C.POINTER(SortedState), I64, I32, P]),
    'jmd_segment_plan': (C.c_int, [C.POINTER(NList), I32, C.POINTER(I32), C.POINTER(I32),
                                   C.POINTER(I64), C.POINTER(I32), C.POINTER(I64)]),
    'jmd_nve_fused_step_segment': (C.c_int, [C.POINTER(Pair), C.POINTER(Space), C.POINTER(NList),
                                             I32, I32, I32, I32, P, P, P, P, F32, I64, I32, P,
                                             I64, F32, P, F32, P, P, C.c_size_t, P, P]),
    'jmd_neighbor_list_build_tiled': (C.c_int, [C.POINTER(NList), P, I64, P, I64, P, P, P, P, P, P,
                                                SZ, P]),
    'jmd_pair_forces_tiled': (C.c_int, [C.POINTER(Pair), C.POINTER(Space), P, P, I64, P, I64, I64,
                                        P, P, P]),
    'jmd_nve_fused_step_tiled': (C.c_int, [C.POINTER(Pair), C.POINTER(Space), P, P, P, F32, P, I64,
                                           P, I64, I64, P, F32, P, F32, P, P]),
    'jmd_pair_force_vjp': (C.c_int, [C.POINTER(Pair), C.POINTER(Space), P, I64, P, I64, P, I64,
                                     I64, P, P, I64, F32, P, I64, P, P, P]),
    'jmd_pair_force_vjp_sparse': (C.c_int, [C.POINTER(Pair), C.POINTER(Space), I32, P, I64, P, I64,
                                            P, I64, I64, P, I64, F32, P, I64, P, P, P]),
    'jmd_nhc_half_step_vjp': (C.c_int, [C.POINTER(Nhc), P, P, I32, P, P, P, P, P]),
    'jmd_langevin_o_step': (C.c_int, [P, I64, I64, I32, P, F32, F32, F32, C.c_uint64, C.c_uint64,
                                      P, P]),
    'jmd_nvt_run': (C.c_int, [C.POINTER(NveSystem), C.POINTER(Nvt), I64, I32, P]),
    'jmd_nvt_run_sorted': (C.c_int, [C.POINTER(NveSystem), C.POINTER(SortedState), C.POINTER(Nvt),
                                     I64, I32, P]),
    'jmd_nve_run_recorded': (C.c_int, [C.POINTER(NveSystem), P, I64, I32, I32, P]),
    'jmd_nve_adjoint_segment': (C.c_int, [C.POINTER(NveSystem), P, I64, I32, I32, P, P, P, P, I32,
                                          P]),
    'jmd_batch_nlist_workspace_bytes': (SZ, [C.POINTER(Batch)]),
    'jmd_batch_neighbor_list_build': (C.c_int, [C.POINTER(Batch), C.POINTER(BatchNList), P, I32,
                                                P]),
    'jmd_batch_skin_check': (C.c_int, [C.POINTER(Batch), C.POINTER(BatchNList), P, F32, P]),
    'jmd_batch_pair_forces': (C.c_int, [C.POINTER(Pair), C.POINTER(Batch), C.POINTER(BatchNList),
                                        P, P, P, P, P]),
    'jmd_batch_kinetic_energy': (C.c_int, [C.POINTER(Batch), P, P, P, F32, P, P, P]),
    'jmd_npt_map': (C.c_int, [I32, P, P, P, P, F32, I64, C.POINTER(Space), F32, F32, P]),
    'jmd_batch_dot_per_system': (C.c_int, [C.POINTER(Batch), P, I64, P, I64, P, P]),
    'jmd_batch_nvt_adjoint_update': (C.c_int, [C.POINTER(Batch), I32, P, P, I64, P, P, F32, F32,
                                               P, P, P, P, P]),
    'jmd_batch_fire_init': (C.c_int, [C.POINTER(BatchSystem), C.POINTER(FireParams), P]),
    'jmd_batch_nve_run': (C.c_int, [C.POINTER(BatchSystem), I64, I32, P]),
    'jmd_batch_fire_run': (C.c_int, [C.POINTER(BatchSystem), C.POINTER(FireParams), I64, I32, P]),
    'jmd_batch_set_launch': (C.c_int, [C.c_int, C.c_int]),
    'jmd_batch_nve_run_recorded': (C.c_int, [C.POINTER(BatchSystem), P, I64, I32, I32, P]),
    'jmd_batch_nve_adjoint_segment': (C.c_int, [C.POINTER(BatchSystem), P, I64, I32, I32, P, P, P,
                                                P, I32, P]),
    'jmd_batch_energy_param_grad': (C.c_int, [C.POINTER(Pair), C.POINTER(Batch),
                                              C.POINTER(BatchNList), P, P, P, P, P]),
    'jmd_batch_nvt_run': (C.c_int, [C.POINTER(BatchSystem), C.POINTER(BatchNvt), I64, I32, P]),
    'jmd_batch_nhc_half_step': (C.c_int, [C.POINTER(Batch), C.POINTER(BatchNvt), P, P, F32, I32,
                                          I32, P, P, P]),
    'jmd_batch_nhc_half_step_vjp': (C.c_int, [C.POINTER(Batch), C.POINTER(Nhc), P, P, I32, P, P,
                                              P, P, P]),
    'jmd_batch_pair_force_vjp': (C.c_int, [C.POINTER(Pair), C.POINTER(Batch),
                                           C.POINTER(BatchNList), P, P, P, F32, P, P, P, P]),
    'jmd_fire_kick_drift': (C.c_int, [P, P, P, P, F32, I64, C.POINTER(Space), P, P]),
    'jmd_fire_workspace_bytes': (SZ, [I64]),
    'jmd_fire_update': (C.c_int, [P, P, I64, I32, P, F32, F32, F32, F32, F32, F32, P, SZ, P]),
    'jmd_force_kick_tiled': (C.c_int, [C.POINTER(Pair), C.POINTER(Space), P, P, P, P, I64, P, I64,
                                       I64, P, F32, P]),
}

_lib = None


class NativeError(RuntimeError):
    pass


def lib():
    """Loads the library (building it first when absent) and binds symbols."""
    global _lib
    if _lib is not None:
        return _lib
    if not LIB_PATH.exists():
        from . import _build
        _build.build()
    L = C.CDLL(str(LIB_PATH))
    for name, (res, args) in SIGNATURES.items():
        fn = getattr(L, name)
        fn.restype = res
        fn.argtypes = args
    _lib = L
    return L


def load_without_gpu():
    """Loads the library for symbol checks on a machine without a GPU."""
    return lib()


def check(rc: int, what: str = ''):
    if rc != 0:
        msg = lib().jmd_last_error().decode(errors='replace')
        raise NativeError(f'{what or "jax_md_gb300"} failed ({rc}): {msg}')


def require_cuda(*tensors):
    if not torch.cuda.is_available():
        raise NativeError('jax_md_gb300 needs a CUDA device: the GB300 kernels are the only '
                          'compute path')
    for t in tensors:
        if t is not None and isinstance(t, torch.Tensor) and not t.is_cuda:
            raise NativeError('jax_md_gb300 operates on CUDA tensors; got a tensor on ' + str(t.device))


def stream_ptr(device=None) -> int:
    return torch.cuda.current_stream(device).cuda_stream


def ptr(t):
    return None if t is None else t.data_ptr()


def row_stride(t: torch.Tensor) -> int:
    """Row stride (in elements) of a 2-D tensor whose rows are contiguous."""
    if t.dim() != 2 or t.stride(1) != 1:
        raise NativeError('expected a [N, d] tensor with contiguous rows')
    return t.stride(0)


_ws_cache = {}


def workspace(nbytes: int, device, key='default') -> torch.Tensor:
    """A cached uint8 device buffer of at least nbytes (per device and key)."""
    k = (str(device), key)
    t = _ws_cache.get(k)
    if t is None or t.numel() < nbytes:
        t = torch.empty(max(nbytes, 256), dtype=torch.uint8, device=device)
        _ws_cache[k] = t
    return t
