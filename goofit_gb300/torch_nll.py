"""The engine's NLL as a differentiable torch function.

`nll(pdf, params)` returns the negative log-likelihood of the PDF's data set at the parameter vector
`params` (a float64 tensor over the PDF's free parameters, in `getParameters()` order), computed by the
generated kernels; its backward pass returns the analytic gradient the same FCN call produced (the sum of
per-event forward tangents), so torch optimisers and higher-level code can drive the fit instead of
MIGRAD.  Parameters without an analytic derivative (an amplitude PDF's efficiency) raise an error.
"""
from __future__ import annotations

import numpy as np
import torch

from .api import GeneralError, PdfBase


class _EngineNLL(torch.autograd.Function):
    @staticmethod
    def forward(ctx, free: torch.Tensor, eng, full: np.ndarray, free_idx: np.ndarray, grad_pos: np.ndarray):
        p = full.copy()
        p[free_idx] = free.detach().cpu().numpy().astype(np.float64)
        value, g = eng.nll_grad(p)
        ctx.save_for_backward(torch.as_tensor(g[grad_pos], dtype=free.dtype, device=free.device))
        return torch.tensor(value, dtype=free.dtype, device=free.device)

    @staticmethod
    def backward(ctx, grad_out):
        (g,) = ctx.saved_tensors
        return grad_out * g, None, None, None, None


def nll(pdf: PdfBase, params: torch.Tensor, precision: str | None = None) -> torch.Tensor:
    """NLL of `pdf` on its data set at the free parameters `params` (autograd-enabled)."""
    if pdf.data is None:
        raise GeneralError("no data set")
    eng, plist = pdf._engine_for(pdf.data, precision)
    full = np.array([v.value - v._blind for v in plist], dtype=np.float64)
    free_idx = np.array([i for i, v in enumerate(plist) if not v.fixed], dtype=np.int64)
    if params.numel() != len(free_idx):
        raise GeneralError(f"expected {len(free_idx)} free parameters, got {params.numel()}")
    slot = {p: s for s, p in enumerate(eng.grad_params)}
    missing = [plist[i].name for i in free_idx if i not in slot]
    if missing:
        raise GeneralError(f"no analytic derivative for {missing}")
    grad_pos = np.array([slot[i] for i in free_idx], dtype=np.int64)
    return _EngineNLL.apply(params.reshape(-1), eng, full, free_idx, grad_pos)


def free_parameters(pdf: PdfBase) -> torch.Tensor:
    """Current values of the free parameters, in the order `nll` expects."""
    return torch.tensor([v.value - v._blind for v in pdf.getParameters() if not v.fixed], dtype=torch.float64)
