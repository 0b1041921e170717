"""GPU tests of the adjoint (backward pass) of the tilted-axis
reconstruction (odt_bpp3d_adjoint on an ODT_GEOM_AFFINE3D plan, the
transpose of k_rotate_3d and of the y-prefilter boundary terms), through
the same torch.autograd.Function as the y-axis path:

* against the dense conjugate-transposed Jacobian of the FP64 oracle
  (odtbrain/_alg3d_bppt.py:374-949 restated), built column by column from
  the oracle's response to every sinogram basis vector;
* the dot-product identity <c, F d> = <F^H c, d> on a larger plan;
* central finite differences (h = 1e-3) along random directions for the
  sinogram and a real per-frequency filter gain.
"""
import numpy as np
import pytest

from oracle import odt_oracle as O
from sino_gen import ellipsoid_phantom_sinogram

pytestmark = pytest.mark.gpu

AXIS = (0.15, float(np.cos(0.25)), float(np.sin(0.25)))


def _rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def torch_dev(cuda_ready):
    import torch
    return torch, cuda_ready


@pytest.mark.parametrize("order", [1, 2, 3])
def test_tilted_adjoint_matches_dense_oracle_jacobian(torch_dev, order):
    torch, dev = torch_dev
    from odtbrain_gb300._alg3d import Backprop3D
    rng = np.random.default_rng(order + 30)
    A, n = 3, 8
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    kw = dict(res=3.0, nm=1.333, tilted_axis=AXIS, intp_order=order,
              padval="edge")
    # dense Jacobian of the (complex-linear) FP64 oracle: column k is the
    # response to the k-th unit sinogram sample
    m = A * n * n
    J = np.empty((n * n * n, m), dtype=np.complex128)
    for k in range(m):
        e = np.zeros(m, dtype=np.complex128)
        e[k] = 1.0
        J[:, k] = O.backpropagate_3d_tilted(e.reshape(A, n, n), angles,
                                            **kw).reshape(-1)
    cot = rng.normal(size=(n, n, n)) + 1j * rng.normal(size=(n, n, n))
    ref = (J.conj().T @ cot.reshape(-1)).reshape(A, n, n)
    rec = Backprop3D((A, n, n), angles, 3.0, 1.333, tilted_axis=AXIS,
                     intp_order=order, input_dtype="complex64", device=dev)
    sino = rng.normal(size=(A, n, n)) + 1j * rng.normal(size=(A, n, n))
    d_s = torch.tensor(sino.astype(np.complex64), device=dev)
    # the forward against the same Jacobian
    vf = rec(d_s).cpu().numpy().reshape(-1)
    assert _rel(vf, J @ sino.reshape(-1)) < 1e-5
    d_c = torch.tensor(cot.astype(np.complex64), device=dev)
    ds, _ = rec.adjoint(d_s, d_c)
    assert _rel(ds.cpu().numpy(), ref) < 2e-5


@pytest.mark.parametrize("padval", ["edge", 0.4])
def test_tilted_adjoint_dot_product_identity(torch_dev, padval):
    torch, dev = torch_dev
    from odtbrain_gb300._alg3d import Backprop3D
    rng = np.random.default_rng(41)
    A, ny, nx = 12, 40, 44
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    rec = Backprop3D((A, ny, nx), angles, 2.5, 1.34, lD=0.5, padval=padval,
                     tilted_axis=AXIS, input_dtype="complex64", device=dev)
    d = torch.tensor((rng.normal(size=(A, ny, nx)) +
                      1j * rng.normal(size=(A, ny, nx))).astype(np.complex64),
                     device=dev)
    c = torch.tensor((rng.normal(size=(nx, ny, nx)) +
                      1j * rng.normal(size=(nx, ny, nx))).astype(np.complex64),
                     device=dev)
    # the linear ramp adds a constant (the end value): difference two
    # evaluations so that only the linear part remains
    Fd = rec(d) - rec(torch.zeros_like(d))
    ds, _ = rec.adjoint(d, c)
    lhs = torch.vdot(c.flatten(), Fd.flatten()).real.item()
    rhs = torch.vdot(ds.flatten(), d.flatten()).real.item()
    assert abs(lhs - rhs) <= 1e-5 * (abs(lhs) + abs(rhs))


def test_tilted_autograd_finite_differences(torch_dev):
    """A=40, 64x64 -> 64^3, axis tilted 0.25 rad; 16 directions for the
    sinogram and for the gain, h=1e-3, through the autograd wrapper."""
    torch, dev = torch_dev
    from odtbrain_gb300.autograd import backpropagate_3d_autograd
    from odtbrain_gb300._alg3d import Backprop3D
    sino, angles = ellipsoid_phantom_sinogram(64, 40, seed=8,
                                              count_range=(2, 5),
                                              semi_range=(4, 16), axis=AXIS)
    rec = Backprop3D(sino.shape, angles, 3.0, 1.333, tilted_axis=AXIS,
                     input_dtype="complex64", device=dev)
    rng = np.random.default_rng(23)
    s = torch.tensor(sino.astype(np.complex64), device=dev)
    g = torch.tensor(rng.uniform(0.8, 1.2, rec.gain_shape())
                     .astype(np.float32), device=dev)
    s_req = s.clone().requires_grad_(True)
    g_req = g.clone().requires_grad_(True)
    vol = backpropagate_3d_autograd(s_req, angles, 3.0, 1.333, gain=g_req,
                                    plan=rec)
    cot = torch.tensor((rng.normal(size=vol.shape) +
                        1j * rng.normal(size=vol.shape))
                       .astype(np.complex64), device=dev)
    loss = torch.vdot(cot.flatten(), vol.flatten()).real
    loss.backward()
    ds, dg = s_req.grad, g_req.grad
    h = 1e-3
    ls, rs, lg, rg = [], [], [], []
    for _ in range(16):
        dirs = torch.tensor((rng.normal(size=s.shape) +
                             1j * rng.normal(size=s.shape))
                            .astype(np.complex64), device=dev)
        fd = (rec.forward_gain(s + h * dirs, g) -
              rec.forward_gain(s - h * dirs, g)) / (2 * h)
        ls.append(torch.vdot(cot.flatten(), fd.flatten()).real.item())
        rs.append(torch.vdot(ds.flatten(), dirs.flatten()).real.item())
        dgr = torch.tensor(rng.normal(size=g.shape).astype(np.float32),
                           device=dev)
        fd = (rec.forward_gain(s, g + h * dgr) -
              rec.forward_gain(s, g - h * dgr)) / (2 * h)
        lg.append(torch.vdot(cot.flatten(), fd.flatten()).real.item())
        rg.append(torch.sum(dg * dgr).item())
    for name, lhs, rhs in (("sino", ls, rs), ("gain", lg, rg)):
        lhs, rhs = np.array(lhs), np.array(rhs)
        rel = np.linalg.norm(lhs - rhs) / np.linalg.norm(rhs)
        worst = np.abs(lhs - rhs).max() / np.sqrt(np.mean(rhs ** 2))
        assert rel < 1e-3 and worst < 1e-2, (name, rel, worst)
