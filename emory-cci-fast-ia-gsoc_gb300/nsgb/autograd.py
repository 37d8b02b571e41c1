"""torch.autograd binding of the differentiable float32 reconstruction (a thin test binding
over the C ABI: nsgb_recon_f32_fwd / nsgb_recon_f32_bwd)."""
from __future__ import annotations

import torch

from . import recon_f32, recon_f32_backward


class ImreconstructF32(torch.autograd.Function):
    """out = imreconstruct(marker, mask) by dilation; the backward scatters the upstream
    gradient to the marker or mask pixel each output value was copied from."""

    @staticmethod
    def forward(ctx, marker: torch.Tensor, mask: torch.Tensor, connectivity: int = 8):
        out, prov = recon_f32(marker, mask, connectivity)
        ctx.save_for_backward(prov)
        return out

    @staticmethod
    def backward(ctx, grad_out: torch.Tensor):
        (prov,) = ctx.saved_tensors
        dmarker, dmask = recon_f32_backward(grad_out.contiguous(), prov)
        return dmarker, dmask, None


def imreconstruct_f32(marker: torch.Tensor, mask: torch.Tensor, connectivity: int = 8) -> torch.Tensor:
    return ImreconstructF32.apply(marker, mask, connectivity)
