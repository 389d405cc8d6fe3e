"""Numerical helpers of jax_md/util.py on torch tensors (util.py:85-112)."""
from __future__ import annotations

from typing import Optional, Sequence, Union

import torch


def safe_mask(mask, fn, operand, placeholder=0):
    """util.py:85-88: fn(operand) where mask holds, placeholder elsewhere;
    fn sees 0 at masked entries, so neither its value nor its gradient is
    evaluated at a singular point."""
    masked = torch.where(mask, operand, torch.zeros_like(operand))
    out = fn(masked)
    return torch.where(mask, out, torch.as_tensor(placeholder, dtype=out.dtype, device=out.device))


def high_precision_sum(X: torch.Tensor, axis: Optional[Union[Sequence[int], int]] = None,
                       keepdims: bool = False) -> torch.Tensor:
    """util.py:91-106: sum at 64-bit precision (int64, complex128 or
    float64), cast back to the input's dtype."""
    if not X.dtype.is_floating_point and not X.dtype.is_complex:
        wide = torch.int64
    elif X.dtype.is_complex:
        wide = torch.complex128
    else:
        wide = torch.float64
    if axis is None:
        s = X.to(wide).sum()
        if keepdims:
            s = s.reshape([1] * X.dim())
    else:
        s = X.to(wide).sum(dim=axis, keepdim=keepdims)
    return s.to(X.dtype)


def maybe_downcast(x):
    """util.py:109-112: float64 tensors stay as they are; anything else
    becomes a float32 tensor."""
    if isinstance(x, torch.Tensor) and x.dtype == torch.float64:
        return x
    return torch.as_tensor(x, dtype=torch.float32)
