"""Differentiable filter + pattern spectrum over a batch of float32 cutouts.

With the component trees held fixed, the direct-rule filtered image and the pattern
spectra are linear in the pixel values: a pixel of the filtered image takes the
level of its nearest surviving node, and a node adds (level - parent level) * area
to one spectrum bin.  A node's level is the value of its level-root pixel, so the
adjoint (dcf_batch_adjoint, a CUDA kernel in the library) scatters each cotangent to
that pixel.  The trees are not stored between forward and backward: backward
rebuilds them from the saved pixels and then runs the adjoint.

    ctx = Context(stream=torch.cuda.current_stream().cuda_stream)
    batch = ctx.batch([(512, 512)] * 256, np.float32, connectivity=8, attribute=14)
    filtered, spectra = filter_and_spectrum(batch, pixels, filter_attr=0, lam=64.0,
                                            spectrum=(14, lvec1, 0, lvec2))

The context must run on the stream torch uses for the surrounding operations (here
the current stream), so that both see each other's work in order.
"""
from __future__ import annotations

import torch

from . import Batch


class FilterSpectrum(torch.autograd.Function):
    """forward(pixels) -> (filtered, spectra); backward rebuilds the trees and runs the adjoint."""

    @staticmethod
    def forward(ctx, pixels: torch.Tensor, batch: Batch, filter_attr: int, lam: float, spectrum, use_graph: bool):
        if pixels.dtype != torch.float32 or not pixels.is_cuda:
            raise TypeError("pixels must be a float32 CUDA tensor")
        flat = pixels.detach().contiguous().view(-1)
        if flat.numel() != batch.n:
            raise ValueError(f"expected {batch.n} pixels, got {flat.numel()}")
        filtered = torch.empty_like(flat)
        n1, n2 = len(spectrum[1]), len(spectrum[3])
        spectra = torch.empty((batch.count, n2, n1), dtype=torch.float64, device=flat.device)
        batch.run(flat, filter_attr, lam, spectrum, use_graph, filtered=filtered, spectra=spectra)
        ctx.batch = batch
        ctx.args = (filter_attr, lam, spectrum, use_graph)
        ctx.shape = pixels.shape
        ctx.save_for_backward(flat)
        return filtered.view_as(pixels), spectra

    @staticmethod
    def backward(ctx, g_filtered, g_spectra):
        (flat,) = ctx.saved_tensors
        batch = ctx.batch
        filter_attr, lam, spectrum, use_graph = ctx.args
        # recompute the trees, attributes and filter targets (no outputs needed)
        batch.run(flat, filter_attr, lam, spectrum, use_graph, want_filtered=False, want_spectra=False)
        v = g_filtered.contiguous().view(-1) if g_filtered is not None else None
        w = g_spectra.contiguous() if g_spectra is not None else None
        if v is not None and v.dtype != torch.float32:
            v = v.float()
        if w is not None and w.dtype != torch.float64:
            w = w.double()
        grad = torch.empty_like(flat)
        batch.adjoint(v, w, out=grad)
        return grad.view(ctx.shape), None, None, None, None, None


def filter_and_spectrum(batch: Batch, pixels: torch.Tensor, filter_attr: int, lam: float, spectrum,
                        use_graph: bool = True):
    """(filtered pixels shaped like `pixels`, spectra[count, n2, n1]) with autograd."""
    return FilterSpectrum.apply(pixels, batch, filter_attr, lam, spectrum, use_graph)
