"""GPU tests of the hand-written adjoint (backward pass) of the y-axis
reconstruction, exposed as odt_bpp3d_adjoint and wrapped in a
torch.autograd.Function (odtbrain_gb300.autograd).

* against torch.autograd through the dense FP64 model of tests/dense_model.py
  (itself pinned to the FP64 oracle on CPU), for the sinogram and for a real
  per-frequency filter gain;
* the dot-product identity <c, F d> = <F^H c, d>;
* central finite differences (h = 1e-3) along 64 random directions at the
  differentiation configuration: A=90, 128x128 sinogram, 128^3 volume, gain
  on the 256x256 padded spectrum grid (the padding rule of
  odtbrain/_alg3d_bpp.py:285-304 turns 128*1.75 into 256).
"""
import numpy as np
import pytest

from sino_gen import ellipsoid_phantom_sinogram

pytestmark = pytest.mark.gpu


def _rel(a, b):
    a = np.asarray(a)
    b = np.asarray(b)
    return np.linalg.norm(a - b) / np.linalg.norm(b)


@pytest.fixture(scope="module")
def torch_dev(cuda_ready):
    import torch
    return torch, cuda_ready


@pytest.mark.parametrize("order", [1, 2, 3])
def test_adjoint_matches_dense_autograd(torch_dev, order):
    torch, dev = torch_dev
    from dense_model import DenseBackprop
    from odtbrain_gb300._alg3d import Backprop3D
    rng = np.random.default_rng(order)
    A, n = 5, 12
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    sino = (rng.normal(0, 0.3, (A, n, n)) + 1j * rng.normal(0, 1, (A, n, n)))
    model = DenseBackprop(angles, n, n, 3.0, 1.333, order=order)
    gshape = (model.geo["lNy"], model.geo["lNx"])
    gain = rng.uniform(0.5, 1.5, gshape)
    cot = rng.normal(size=(n, n, n)) + 1j * rng.normal(size=(n, n, n))

    s64 = torch.tensor(sino, requires_grad=True)
    g64 = torch.tensor(gain, requires_grad=True)
    vol = model(s64, g64)
    ds_ref, dg_ref = torch.autograd.grad(vol, [s64, g64],
                                         grad_outputs=torch.tensor(cot))

    rec = Backprop3D((A, n, n), angles, 3.0, 1.333, intp_order=order,
                     input_dtype="complex64", device=dev)
    d_s = torch.tensor(sino.astype(np.complex64), device=dev)
    d_g = torch.tensor(gain.astype(np.float32), device=dev)
    # forward with gain against the dense model
    vf = rec.forward_gain(d_s, d_g).cpu().numpy()
    assert _rel(vf, vol.detach().numpy()) < 1e-5
    d_c = torch.tensor(cot.astype(np.complex64), device=dev)
    ds, dg = rec.adjoint(d_s, d_c, gain=d_g, need_sino=True, need_gain=True)
    assert _rel(ds.cpu().numpy(), ds_ref.numpy()) < 2e-5
    assert _rel(dg.cpu().numpy(), dg_ref.numpy()) < 2e-5


@pytest.mark.parametrize("order", [1, 2])
def test_angle_gain_adjoint_matches_dense_autograd(torch_dev, order):
    """Per-angle complex gains (the learned filter's output): forward and
    both gradients against autograd through the dense FP64 model."""
    torch, dev = torch_dev
    from dense_model import DenseBackprop
    from odtbrain_gb300._alg3d import Backprop3D
    rng = np.random.default_rng(10 + order)
    A, ny, nx = 6, 10, 12
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    sino = (rng.normal(0, 0.3, (A, ny, nx)) +
            1j * rng.normal(0, 1, (A, ny, nx)))
    model = DenseBackprop(angles, ny, nx, 2.7, 1.333, order=order)
    gshape = (A, model.geo["lNy"], model.geo["lNx"])
    ag = (rng.uniform(0.5, 1.5, gshape) +
          1j * rng.uniform(-0.5, 0.5, gshape))
    cot = (rng.normal(size=(nx, ny, nx)) +
           1j * rng.normal(size=(nx, ny, nx)))
    s64 = torch.tensor(sino, requires_grad=True)
    a64 = torch.tensor(ag, requires_grad=True)
    vol = model(s64, angle_gain=a64)
    ds_ref, da_ref = torch.autograd.grad(vol, [s64, a64],
                                         grad_outputs=torch.tensor(cot))
    rec = Backprop3D((A, ny, nx), angles, 2.7, 1.333, intp_order=order,
                     input_dtype="complex64", device=dev)
    d_s = torch.tensor(sino.astype(np.complex64), device=dev)
    d_a = torch.tensor(ag.astype(np.complex64), device=dev)
    vf = rec.forward_gain(d_s, angle_gain=d_a).cpu().numpy()
    assert _rel(vf, vol.detach().numpy()) < 1e-5
    d_c = torch.tensor(cot.astype(np.complex64), device=dev)
    ds, dg, da = rec.adjoint(d_s, d_c, angle_gain=d_a, need_sino=True,
                             need_angle_gain=True)
    assert dg is None
    assert _rel(ds.cpu().numpy(), ds_ref.numpy()) < 2e-5
    assert _rel(da.cpu().numpy(), da_ref.numpy()) < 2e-5


@pytest.mark.parametrize("padval", ["edge", 0.7])
@pytest.mark.parametrize("ny,padding", [(40, (True, True)),
                                        (1, (True, True)),
                                        (1, (False, False))])
def test_adjoint_dot_product_identity(torch_dev, padval, ny, padding):
    """Also for one detector row: padded (pitch-1 slab, one output per
    thread in the resampling) and unpadded (the fused single-row stage)."""
    torch, dev = torch_dev
    from odtbrain_gb300._alg3d import Backprop3D
    rng = np.random.default_rng(9)
    A, nx = 14, 48
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    rec = Backprop3D((A, ny, nx), angles, 2.5, 1.34, lD=1.0, padval=padval,
                     padding=padding, input_dtype="complex64", device=dev)
    d = torch.tensor((rng.normal(size=(A, ny, nx)) +
                      1j * rng.normal(size=(A, ny, nx))).astype(np.complex64),
                     device=dev)
    c = torch.tensor((rng.normal(size=(nx, ny, nx)) +
                      1j * rng.normal(size=(nx, ny, nx))).astype(np.complex64),
                     device=dev)
    if padval != "edge":
        # the linear ramp adds a constant (the end value); difference two
        # evaluations so that only the linear part remains
        zero = torch.zeros_like(d)
        Fd = rec(d) - rec(zero)
    else:
        Fd = rec(d)
    ds, _ = rec.adjoint(d, c)
    lhs = torch.vdot(c.flatten(), Fd.flatten()).real.item()
    rhs = torch.vdot(ds.flatten(), d.flatten()).real.item()
    assert abs(lhs - rhs) <= 1e-5 * (abs(lhs) + abs(rhs))


def test_finite_differences_differentiation_config(torch_dev):
    """A=90, 128x128 -> 128^3; 64 random directions, h=1e-3."""
    torch, dev = torch_dev
    from odtbrain_gb300.autograd import backpropagate_3d_autograd
    from odtbrain_gb300._alg3d import Backprop3D
    sino, angles = ellipsoid_phantom_sinogram(128, 90, seed=5,
                                              count_range=(2, 6),
                                              semi_range=(6, 30))
    rec = Backprop3D(sino.shape, angles, 3.0, 1.333,
                     input_dtype="complex64", device=dev)
    assert rec.gain_shape() == (256, 256)
    rng = np.random.default_rng(17)
    s = torch.tensor(sino.astype(np.complex64), device=dev)
    g = torch.tensor(rng.uniform(0.8, 1.2, rec.gain_shape())
                     .astype(np.float32), device=dev)
    torch.cuda.reset_peak_memory_stats(dev)
    s_req = s.clone().requires_grad_(True)
    g_req = g.clone().requires_grad_(True)
    vol = backpropagate_3d_autograd(s_req, angles, 3.0, 1.333, gain=g_req,
                                    plan=rec)
    cot = torch.tensor((rng.normal(size=vol.shape) +
                        1j * rng.normal(size=vol.shape))
                       .astype(np.complex64), device=dev)
    loss = torch.vdot(cot.flatten(), vol.flatten()).real
    loss.backward()
    peak = torch.cuda.max_memory_allocated(dev)
    print("\nforward+backward peak device memory: %.1f MiB" % (peak / 2**20))
    ds = s_req.grad
    dg = g_req.grad
    h = 1e-3
    ls, rs, lg, rg = [], [], [], []
    for k in range(64):
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
    # the 64 directional derivatives: finite differences (FP32 forward,
    # h=1e-3) against the adjoint; a single projection can be near zero,
    # so errors are measured against the rms of the 64 values
    for name, lhs, rhs in (("sino", ls, rs), ("gain", lg, rg)):
        lhs, rhs = np.array(lhs), np.array(rhs)
        rel = np.linalg.norm(lhs - rhs) / np.linalg.norm(rhs)
        worst = np.abs(lhs - rhs).max() / np.sqrt(np.mean(rhs ** 2))
        print("finite differences (%s): rel-L2 %.2e, worst %.2e of rms" %
              (name, rel, worst))
        assert rel < 1e-3 and worst < 1e-2, name
