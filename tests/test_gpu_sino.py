"""GPU parity of the sinogram preparation (odtbrain_gb300.sinogram_as_rytov /
sinogram_as_radon / align_unwrapped / unwrap_frames) against the
reference's golden vectors, reference-made fixtures and the CPU oracle
(oracle/unwrap_oracle.py).

Tolerances: the unwrapped phase is the wrapped phase plus whole turns, so
with identical turns the only differences come from the elementwise
angle / log (CUDA vs NumPy, within a few ulp): rtol 1e-12 for FP64 data,
1e-5 for FP32 data.  The unwrapping itself (given identical wrapped
phases) is compared bit for bit."""
import json
import os

import numpy as np
import pytest

from oracle import unwrap_oracle as uo

pytestmark = pytest.mark.gpu
TWOPI = 2 * np.pi
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def sino_fix():
    with np.load(os.path.join(GOLDEN, "reference_sino.npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="module")
def prep(cuda_ready):
    import odtbrain_gb300
    from odtbrain_gb300 import _prepare_sino
    return odtbrain_gb300, _prepare_sino


def processing_sino(rytov=False):
    ln, a = 10, 2
    sino = np.arange(ln * ln * a).reshape(a, ln, ln) / (ln * ln * a) * \
        np.exp(1j * np.arange(ln * ln * a).reshape(a, ln, ln))
    if rytov:
        sino[0, 0, 0] = .1
    return sino


def negative_modulo_rest(a, b):
    q = np.array(a / b, dtype=int)
    r = a - b * q
    wrong = np.where(np.abs(r) > b / 2)
    r[wrong] -= b * np.sign(r[wrong])
    return r


def test_sino_rytov_golden(prep, sino_fix):
    """tests/test_processing.py:109-137 of the reference, on the GPU."""
    odt, _ = prep
    ryt = odt.sinogram_as_rytov(processing_sino(rytov=True))
    assert ryt.dtype == np.complex128
    if ryt.imag.min() > TWOPI:
        ryt.imag -= TWOPI
    assert np.allclose(np.array(ryt).flatten().view(float),
                       sino_fix["zip_test_sino_rytov"])
    s = processing_sino(rytov=True)
    for two, three in ((s[:, :, 0], ryt[:, :, 0]), (s[:, 0, :], ryt[:, 0, :])):
        d = odt.sinogram_as_rytov(two) - three
        assert np.allclose(0, d.real, atol=1e-6)
        assert np.allclose(0, negative_modulo_rest(d.imag, TWOPI), atol=1e-6)


def test_sino_radon_golden(prep, sino_fix):
    """tests/test_processing.py:78-106 of the reference, on the GPU."""
    odt, _ = prep
    rad = odt.sinogram_as_radon(processing_sino())
    if rad.min() > TWOPI:
        rad -= TWOPI
    assert np.allclose(rad.ravel(), sino_fix["zip_test_sino_radon"])
    s = processing_sino()
    for two, three in ((s[:, :, 0], rad[:, :, 0]), (s[:, 0, :], rad[:, 0, :])):
        d = odt.sinogram_as_radon(two) - three
        assert np.allclose(0, negative_modulo_rest(d, TWOPI), atol=1e-6)


def test_matches_reference_runs(prep, sino_fix):
    """Outputs of the reference's own sinogram_as_rytov / _radon (3D cases
    with the oracle's unwrap inside)."""
    odt, _ = prep
    names = sorted({k.split("__")[0] for k in sino_fix if "__" in k})
    assert len(names) == 13
    for n in names:
        sino = sino_fix[n + "__sino"]
        kw = json.loads(str(sino_fix[n + "__kw"]))
        out = sino_fix[n + "__out"]
        if kw["kind"] == "rytov":
            args = {}
            if n + "__u0" in sino_fix:
                u0 = sino_fix[n + "__u0"]
                args["u0"] = float(u0) if u0.ndim == 0 else u0
            got = odt.sinogram_as_rytov(sino, align=kw["align"], **args)
        else:
            got = odt.sinogram_as_radon(sino, align=kw["align"])
        assert got.dtype == out.dtype, n
        tol = 1e-5 if out.dtype in (np.complex64, np.float32) else 1e-12
        np.testing.assert_allclose(got, out, rtol=tol, atol=tol, err_msg=n)


def _noisy_frames(rng, A, H, W, noise):
    y, x = np.mgrid[:H, :W]
    out = np.empty((A, H, W))
    for a in range(A):
        cy, cx = rng.uniform(0.3, 0.7) * H, rng.uniform(0.3, 0.7) * W
        r = rng.uniform(0.15, 0.4) * max(H, W)
        ph = rng.uniform(3, 20) * np.exp(-((y - cy) ** 2 + (x - cx) ** 2)
                                         / r ** 2)
        out[a] = ph + rng.normal(0, noise, (H, W))
    return np.angle(np.exp(1j * out))


def _smooth_frames(rng, A, H, W):
    """Residue-free wrapped frames: Gaussian phase bumps whose gradient
    stays below 1.5 rad per pixel."""
    y, x = np.mgrid[:H, :W]
    out = np.empty((A, H, W))
    for a in range(A):
        cy, cx = rng.uniform(0.3, 0.7) * H, rng.uniform(0.3, 0.7) * W
        r = rng.uniform(0.3, 0.5) * max(H, W)
        amp = rng.uniform(3, 1.5 * r / 0.86)
        out[a] = amp * np.exp(-((y - cy) ** 2 + (x - cx) ** 2) / r ** 2) \
            + rng.normal(0, 0.01, (H, W))
    return np.angle(np.exp(1j * out))


def _object_frames(rng, A, H, W, background=0.7):
    """Wrapped frames of an object inside a flat background phase (the
    sinogram of a sample in a medium): Gaussian bumps inside the central
    region, gradient below 1.3 rad per pixel, so the frame corners follow
    the background from angle to angle."""
    y, x = np.mgrid[:H, :W]
    out = np.empty((A, H, W))
    for a in range(A):
        cy = rng.uniform(0.4, 0.6) * H
        cx = rng.uniform(0.4, 0.6) * W
        r = rng.uniform(0.1, 0.18) * min(H, W)
        amp = rng.uniform(2, 1.3 * r / 0.86)
        out[a] = background + amp * np.exp(-((y - cy) ** 2 + (x - cx) ** 2)
                                           / r ** 2) \
            + rng.normal(0, 0.01, (H, W))
    return np.angle(np.exp(1j * out))


@pytest.mark.parametrize("shape,noise", [
    ((6, 17, 23), 0.05), ((5, 24, 31), 0.9), ((4, 32, 32), 2.5),
    ((3, 1, 19), 0.3), ((3, 19, 1), 0.3), ((2, 2, 2), 1.0), ((2, 3, 3), 2.0),
    ((1, 1, 1), 0.0), ((2, 64, 80), 1.2)])
def test_unwrap_frames_bit_exact(prep, shape, noise):
    """Same wrapped FP64 phases in: the GPU spanning tree equals the
    oracle's Kruskal tree (residues included), with the first-edge anchor."""
    _, ps = prep
    rng = np.random.default_rng(hash(shape) % 1000 + int(noise * 10))
    w = _noisy_frames(rng, *shape, noise)
    got = ps.unwrap_frames(w)
    for a in range(shape[0]):
        ref = uo.unwrap_2d(w[a], anchor="first_edge")
        assert np.array_equal(got[a], ref), (shape, noise, a)


def test_unwrap_frames_float32_and_tensor(prep):
    import torch
    _, ps = prep
    rng = np.random.default_rng(7)
    w = _noisy_frames(rng, 3, 21, 26, 0.7).astype(np.float32)
    got = ps.unwrap_frames(torch.from_numpy(w).cuda())
    assert got.is_cuda and got.dtype == torch.float32
    for a in range(3):
        ref = uo.unwrap_2d(w[a], anchor="first_edge").astype(np.float32)
        assert np.array_equal(got[a].cpu().numpy(), ref)
    single = ps.unwrap_frames(w[0])
    assert single.shape == (21, 26)
    assert np.array_equal(single, got[0].cpu().numpy())


def test_reference_head_anchor_modulo_whole_turns(prep):
    """Against the reference's anchor (the pixel heading the final group)
    the unwrapped frames differ by at most one whole-turn constant per
    frame (the offset the reference's own tests treat as platform-dependent,
    tests/test_processing.py:83-90, and align_unwrapped removes)."""
    _, ps = prep
    rng = np.random.default_rng(11)
    w = _smooth_frames(rng, 8, 40, 36)
    got = ps.unwrap_frames(w)
    for a in range(8):
        d = got[a] - uo.unwrap_2d(w[a])
        k = np.round(d / TWOPI)
        assert len(np.unique(k)) == 1
        np.testing.assert_allclose(d, TWOPI * k, rtol=0, atol=1e-12)


@pytest.mark.parametrize("dtype", [np.complex64, np.complex128])
@pytest.mark.parametrize("align", [True, False])
def test_rytov_3d_vs_oracle(prep, dtype, align):
    odt, _ = prep
    rng = np.random.default_rng(5)
    A, H, W = 7, 38, 43
    ph = _object_frames(rng, A, H, W)
    amp = np.exp(0.1 * rng.standard_normal((A, H, W)))
    u = (amp * np.exp(1j * ph)).astype(dtype)
    got = odt.sinogram_as_rytov(u, align=align)
    ref = uo.sinogram_as_rytov(u, align=align, anchor="first_edge")
    assert got.dtype == ref.dtype == dtype
    tol = 1e-5 if dtype == np.complex64 else 1e-12
    np.testing.assert_allclose(got, ref, rtol=tol, atol=tol)


def test_rytov_tensor_in_tensor_out(prep):
    import torch
    odt, _ = prep
    rng = np.random.default_rng(9)
    u = np.exp(1j * _object_frames(rng, 5, 26, 30)).astype(np.complex64)
    t = torch.from_numpy(u).cuda()
    got = odt.sinogram_as_rytov(t)
    assert got.is_cuda and got.dtype == torch.complex64
    np.testing.assert_allclose(got.cpu().numpy(), odt.sinogram_as_rytov(u),
                               rtol=0, atol=0)


def test_align_unwrapped_vs_oracle(prep):
    """Per-angle whole-turn steps planted in an unwrapped sinogram are
    removed exactly as the reference's align_unwrapped removes them."""
    _, ps = prep
    rng = np.random.default_rng(13)
    for shape in ((40, 24), (30, 12, 17)):
        base = np.cumsum(rng.normal(0, 0.05, shape), axis=0) + 7.0
        steps = TWOPI * rng.integers(-2, 3, shape[0])
        s = base + steps.reshape((-1,) + (1,) * (len(shape) - 1))
        for dt in (np.float64, np.float32):
            a = s.astype(dt)
            ref = a.copy()
            uo.align_unwrapped(ref)
            got = a.copy()
            ps.align_unwrapped(got)
            tol = 0 if dt == np.float64 else 1e-6
            np.testing.assert_allclose(got, ref, rtol=tol, atol=tol)


def test_zero_amplitude_gives_reference_nan_pattern(prep):
    odt, _ = prep
    s = np.exp(1j * np.linspace(0, 3, 30)).reshape(3, 10).astype(np.complex128)
    s[1, 4] = 0
    got = odt.sinogram_as_rytov(s, align=False)
    ref = uo.sinogram_as_rytov(s, align=False)
    np.testing.assert_array_equal(np.isnan(got.imag), np.isnan(ref.imag))
    np.testing.assert_array_equal(np.isinf(got.real), np.isinf(ref.real))
    fin = np.isfinite(ref.real)
    np.testing.assert_allclose(got.real[fin], ref.real[fin], rtol=0,
                               atol=1e-15)


def test_errors(prep):
    odt, ps = prep
    with pytest.raises(ValueError):
        odt.sinogram_as_rytov(np.ones(5, dtype=complex))
    with pytest.raises(NotImplementedError):
        odt.sinogram_as_rytov(np.ones((2, 2, 2, 2), dtype=complex))
    with pytest.raises(ValueError):
        odt.sinogram_as_rytov(np.ones((3, 4), dtype=complex),
                              u0=np.ones(5))
    with pytest.raises(ValueError):
        ps.align_unwrapped(np.ones((3, 4), dtype=np.int32))


def test_large_frames_property(prep):
    """200 frames of 256 x 256 (the benchmark sinogram's size): the
    unwrapped phase of residue-free frames is the true phase plus one whole
    turn count per frame."""
    import torch
    odt, ps = prep
    A, H, W = 200, 256, 256
    y, x = torch.meshgrid(torch.arange(H, device="cuda", dtype=torch.float64),
                          torch.arange(W, device="cuda", dtype=torch.float64),
                          indexing="ij")
    a = torch.arange(A, device="cuda", dtype=torch.float64)[:, None, None]
    true = 30.0 * torch.exp(-((y - 128 - 40 * torch.cos(a * 0.03)) ** 2
                              + (x - 128) ** 2) / 2500.0)
    w = torch.atan2(torch.sin(true), torch.cos(true))
    got = ps.unwrap_frames(w)
    k = torch.round((got - true) / TWOPI)
    kk = k.reshape(A, -1)
    assert torch.all(kk == kk[:, :1])
    assert torch.allclose(got - TWOPI * k, true, atol=1e-9)
