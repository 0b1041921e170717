"""Differentiable 3D backpropagation.

``backpropagate_3d_autograd`` wraps the GPU reconstruction (rotation about
y, odtbrain/_alg3d_bpp.py:84-555, or about a tilted axis,
odtbrain/_alg3d_bppt.py:374-949) in a ``torch.autograd.Function``
whose backward pass is the hand-written adjoint of the CUDA pipeline
(``odt_bpp3d_adjoint``): gradients flow to the complex sinogram and to an
optional real per-frequency filter gain of the padded spectrum grid
(shape (lNy, lNx), FFT order).  Nothing of the forward pass is stored: the
backward recomputes the spectra it needs from the saved sinogram.

Gradient convention: PyTorch's -- for the complex sinogram the gradient is
the adjoint (conjugate transpose) of the linear map applied to the volume
cotangent; the real gain receives the real part of its adjoint.
"""
import numpy as np
import torch

from ._alg3d import Backprop3D


class _BackpropagateFn(torch.autograd.Function):
    @staticmethod
    def forward(ctx, sino, gain, rec):
        vol = rec.forward_gain(sino.contiguous(), gain)
        ctx.rec = rec
        ctx.save_for_backward(sino, gain if gain is not None
                              else torch.empty(0))
        ctx.has_gain = gain is not None
        return vol

    @staticmethod
    def backward(ctx, grad_vol):
        sino, gain = ctx.saved_tensors
        gain = gain if ctx.has_gain else None
        need_s = ctx.needs_input_grad[0]
        need_g = ctx.has_gain and ctx.needs_input_grad[1]
        if not (need_s or need_g):
            return None, None, None
        grad_vol = grad_vol.to(torch.complex64).contiguous()
        sg, gg = ctx.rec.adjoint(sino.contiguous(), grad_vol, gain=gain,
                                 need_sino=need_s, need_gain=need_g)
        return sg, gg, None


def backpropagate_3d_autograd(sino, angles, res, nm, lD=0, gain=None,
                              weight_angles=True, padding=(True, True),
                              padfac=1.75, padval="edge", intp_order=2,
                              plan=None, tilted_axis=None):
    """Differentiable ``backpropagate_3d`` (or, with ``tilted_axis``,
    ``backpropagate_3d_tilted``) for a complex64 CUDA sinogram tensor
    (A, Ny, Nx).  ``gain``: optional float32 CUDA tensor of the padded
    spectrum shape multiplying the filter.  ``plan``: a prepared
    :class:`Backprop3D` to reuse (built from the arguments otherwise).
    Spline orders 0..3.  Returns the complex64 volume (Nx, Ny, Nx), indexed
    [z, y, x]."""
    if plan is None:
        plan = Backprop3D(tuple(sino.shape), np.asarray(angles), res, nm,
                          lD=lD, tilted_axis=tilted_axis,
                          weight_angles=weight_angles,
                          padding=padding, padfac=padfac, padval=padval,
                          intp_order=intp_order, input_dtype="complex64",
                          device=sino.device)
    return _BackpropagateFn.apply(sino, gain, plan)
