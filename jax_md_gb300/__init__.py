"""GB300-native short-range molecular dynamics with JAX MD's API.

Submodules mirror jax_md: ``space``, ``partition``, ``smap``, ``energy``,
``quantity``, ``simulate``, ``minimize``.  All compute runs in the sm_103a
CUDA library ``libjaxmd_gb300.so`` (C ABI in include/jax_md_gb300.h);
PyTorch provides device memory and streams.
"""
from . import space, partition, smap, energy, quantity, simulate, minimize, adjoint, batch, util  # noqa: F401

__all__ = ["space", "partition", "smap", "energy", "quantity", "simulate", "minimize", "adjoint", "batch"]
