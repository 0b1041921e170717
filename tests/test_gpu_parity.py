"""GPU parity tests: the CUDA path (through the C ABI) against the FP64
oracle, the reference's golden vectors and fixtures made by the unmodified
reference.

Tolerances (FP32 GPU arithmetic vs FP64 reference), written per test:
  * relative L2 error  <= 1e-5   (the stated target), and
  * max |error| <= 1e-5 * max|reference| (single worst voxel).
"""
import multiprocessing as mp

import numpy as np
import pytest

from conftest import reference_c1, reference_cases
from oracle import odt_oracle as O
from sino_gen import (cutout, ellipsoid_phantom_sinogram, gauss_sino_3d,
                      gauss_sino_3d_tilted, parameter_sets)

pytestmark = pytest.mark.gpu

REL_L2 = 1e-5
MAX_REL = 1e-5


def errs(got, ref):
    got = np.asarray(got)
    ref = np.asarray(ref)
    rel = np.linalg.norm(got - ref) / max(np.linalg.norm(ref), 1e-300)
    mx = np.abs(got - ref).max() / max(np.abs(ref).max(), 1e-300)
    return rel, mx


def assert_close(got, ref, rel_l2=REL_L2, max_rel=MAX_REL, what=""):
    assert got.shape == ref.shape, (what, got.shape, ref.shape)
    rel, mx = errs(got, ref)
    assert rel <= rel_l2 and mx <= max_rel, \
        "%s rel-L2 %.3e (<= %.1e), max %.3e (<= %.1e)" % (
            what, rel, rel_l2, mx, max_rel)


@pytest.fixture(scope="module")
def odt(cuda_ready):
    import odtbrain_gb300
    return odtbrain_gb300


def test_golden_backprop_phase(odt, golden):
    """test_alg3d_bpp.py:30-42: padval=0 (linear ramp), complex result."""
    sino, angles = gauss_sino_3d()
    r = [cutout(odt.backpropagate_3d(sino, angles, padval=0, dtype=float,
                                     **p)) for p in parameter_sets(2)]
    data = np.array(r).flatten().view(float)
    ref = golden["reference_zips"]["test_3d_backprop_phase"]
    assert_close(data, ref, what="phase")
    # the reference's own FP32-vs-FP64 bound (test_alg3d_bpp.py:101-113)
    assert np.allclose(data, ref, atol=6e-7 * 4, rtol=0)


def test_golden_backprop_nopadreal(odt, golden):
    """test_alg3d_bpp.py:45-62: no padding (22-point DFTs), real part."""
    sino, angles = gauss_sino_3d()
    r = [cutout(odt.backpropagate_3d(sino, angles, padding=(False, False),
                                     dtype=float, onlyreal=True, **p))
         for p in parameter_sets(2)]
    data = np.array(r).flatten().view(float)
    ref = golden["reference_zips"]["test_3d_backprop_nopadreal"]
    assert_close(data, ref, what="nopadreal")


def test_reference_cases(odt, golden):
    for name, sino, angles, kw, out in reference_cases(golden):
        fn = (odt.backpropagate_3d_tilted if name.startswith("bppt")
              else odt.backpropagate_3d)
        got = fn(sino, angles, **kw)
        assert got.dtype == out.dtype, name
        assert_close(got, out, what=name)


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("kind", ["y", "tilted"])
def test_orders_vs_oracle(odt, order, kind):
    rng = np.random.default_rng(order * 7 + (kind == "y"))
    A, ny, nx = 10, 18, 20
    sino = (rng.normal(0, .1, (A, ny, nx))
            + 1j * rng.normal(0, .5, (A, ny, nx)))
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    kw = dict(res=3.0, nm=1.333, intp_order=order, padval="edge")
    if kind == "y":
        ref = O.backpropagate_3d(sino, angles, **kw)
        got = odt.backpropagate_3d(sino, angles, **kw)
    else:
        ax = [0.1, 1.0, 0.25]
        ref = O.backpropagate_3d_tilted(sino, angles, tilted_axis=ax, **kw)
        got = odt.backpropagate_3d_tilted(sino, angles, tilted_axis=ax, **kw)
    # order 0 is nearest-neighbour: a voxel's value jumps where its
    # coordinate crosses a half-integer; FP32 filtering does not move
    # coordinates (FP64 geometry), so the bound stays the same
    assert_close(got, ref, what="order %d %s" % (order, kind))


@pytest.mark.parametrize("kind", ["y", "tilted"])
@pytest.mark.parametrize("padding", [(True, True), (False, False)])
def test_single_detector_row(odt, kind, padding):
    """A sinogram of one detector row (A, 1, N): the slab is stored without
    a y pitch and resampled with one output per thread (y axis) or by the
    tilted kernel; unpadded, the column transforms are the identity and run
    inside the row stage."""
    rng = np.random.default_rng(11 + padding[0])
    A, nx = 12, 24
    shape = (A, 1, nx)
    sino = np.exp(1j * rng.normal(0, .4, shape) + rng.normal(0, .05, shape))
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    kw = dict(res=3.0, nm=1.333, padding=padding, padval="edge")
    if kind == "y":
        ref = O.backpropagate_3d(sino, angles, **kw)
        got = odt.backpropagate_3d(sino, angles, **kw)
    else:
        # the affine path about y itself: a tilted axis maps every output
        # off the single row (the reference gives zeros there)
        ax = [0.0, 1.0, 0.0]
        ref = O.backpropagate_3d_tilted(sino, angles, tilted_axis=ax, **kw)
        got = odt.backpropagate_3d_tilted(sino, angles, tilted_axis=ax, **kw)
    assert np.abs(ref).max() > 0
    assert_close(got, ref, what="%s %s" % (kind, padding))


@pytest.mark.parametrize("shape,padding,padval", [
    ((6, 16, 16), (True, True), "edge"),      # padded to 64
    ((5, 64, 64), (False, False), "edge"),    # 64-point Stockham, unpadded
    ((5, 30, 24), (False, False), "edge"),    # generic DFT both axes
    ((4, 70, 40), (True, True), 0.5),         # 128 x 128 padded, ramp
    ((4, 9, 37), (True, True), 2j * np.pi),   # complex ramp end value
])
def test_padding_and_sizes(odt, shape, padding, padval):
    rng = np.random.default_rng(sum(shape))
    A, ny, nx = shape
    sino = np.exp(1j * rng.normal(0, .4, shape) + rng.normal(0, .05, shape))
    # distinct modulo pi: symmetric sets make the angle weights 0/0, in the
    # reference as here
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    kw = dict(res=2.5, nm=1.335, lD=1.5, padding=padding, padval=padval)
    ref = O.backpropagate_3d(sino, angles, **kw)
    got = odt.backpropagate_3d(sino, angles, **kw)
    assert_close(got, ref, what=str(shape))


@pytest.mark.parametrize("order", [2, 4])
@pytest.mark.parametrize("shape,padding", [
    ((5, 30, 24), (False, False)),   # generic DFT columns
    ((5, 64, 64), (False, False)),   # 64-point Stockham columns, no crop
    ((4, 70, 40), (True, True)),     # 128-point columns cropped to 70
])
def test_tilted_sizes_and_orders(odt, shape, padding, order):
    """Tilted plans whose y crop is not the centred half: the column stage
    stores the crop raw with the y-line samples around its ends, and the
    row stage adds the y-prefilter boundary terms (one pole at order 2, two
    at order 4), for every column line type."""
    rng = np.random.default_rng(sum(shape) + order)
    A = shape[0]
    sino = np.exp(1j * rng.normal(0, .4, shape) + rng.normal(0, .05, shape))
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    ax = [0.15, 1.0, -0.2]
    kw = dict(res=2.5, nm=1.335, lD=1.5, padding=padding, padval="edge",
              intp_order=order)
    ref = O.backpropagate_3d_tilted(sino, angles, tilted_axis=ax, **kw)
    got = odt.backpropagate_3d_tilted(sino, angles, tilted_axis=ax, **kw)
    assert_close(got, ref, what="%s order %d" % (shape, order))


def test_onlyreal_matches_real_part(odt):
    """test_alg3d_bpp.py:77-98."""
    sino, angles = gauss_sino_3d(Nx=10, Ny=10)
    for p in parameter_sets(2):
        c = odt.backpropagate_3d(sino, angles, padval=0, dtype=float, **p)
        r = odt.backpropagate_3d(sino, angles, padval=0, dtype=float,
                                 onlyreal=True, **p)
        assert r.dtype == np.float64
        assert np.allclose(c.real, r, rtol=0, atol=1e-7 * np.abs(c).max())


def test_float32_dtype(odt):
    sino, angles = gauss_sino_3d()
    p = parameter_sets(1)[0]
    f32 = odt.backpropagate_3d(sino, angles, padval=0, dtype=np.float32, **p)
    f64 = odt.backpropagate_3d(sino, angles, padval=0, dtype=float, **p)
    assert f32.dtype == np.complex64 and f64.dtype == np.complex128
    assert np.array_equal(f32.astype(np.complex128), f64)


@pytest.mark.parametrize("fn", ["backpropagate_3d", "backpropagate_3d_tilted"])
def test_save_memory_and_copy(odt, fn):
    """test_save_memory.py and test_copy.py: identical results."""
    sino, angles = gauss_sino_3d(Nx=10, Ny=10)
    p = parameter_sets(1)[0]
    f = getattr(odt, fn)
    a = f(sino, angles, padval=0, save_memory=False, **p)
    b = f(sino, angles, padval=0, save_memory=True, **p)
    assert np.array_equal(a, b)
    s2 = sino.copy()
    c = f(s2, angles, padval=0, copy=False, **p)
    assert np.allclose(a, c, rtol=1e-6, atol=1e-7 * np.abs(a).max())
    # copy=False overwrote the caller's array with the weighted sinogram
    from odtbrain_gb300.util import compute_angle_weights_1d
    w = compute_angle_weights_1d(angles).reshape(-1, 1, 1)
    assert np.allclose(s2, sino * w)


@pytest.mark.parametrize("fn", ["backpropagate_3d", "backpropagate_3d_tilted"])
def test_even_weights(odt, fn):
    """test_weighting.py: uniform angles give weights 1."""
    sino, angles = gauss_sino_3d()
    p = parameter_sets(1)[0]
    f = getattr(odt, fn)
    a = f(sino, angles, weight_angles=False, **p)
    b = f(sino, angles, weight_angles=True, **p)
    assert np.allclose(a, b, rtol=0, atol=1e-6 * np.abs(a).max())


@pytest.mark.parametrize("fn", ["backpropagate_3d", "backpropagate_3d_tilted"])
def test_counters(odt, fn):
    """test_counters.py:63-90."""
    sino, angles = gauss_sino_3d(Nx=10, Ny=10)
    p = parameter_sets(1)[0]
    jmc = mp.Value("i", 0)
    jmm = mp.Value("i", 0)
    getattr(odt, fn)(sino, angles, padval=0, count=jmc, max_count=jmm, **p)
    assert jmc.value == jmm.value
    assert jmc.value != 0


def test_tilted_default_axis_equals_plain(odt):
    """test_alg3d_bppt.py:10-50."""
    sino, angles = gauss_sino_3d()
    for p in parameter_sets(2):
        for pv in (0, "edge"):
            a = odt.backpropagate_3d(sino, angles, padval=pv, **p)
            b = odt.backpropagate_3d_tilted(sino, angles, padval=pv, **p)
            assert np.allclose(a, b, rtol=0, atol=2e-6 * np.abs(a).max())


def test_tilted_plane_rotation_soft(odt):
    """test_alg3d_bppt.py:53-86 (the reference's soft tolerance)."""
    p = parameter_sets(1)[0]
    results = []
    for angz in [1.1, 0.0, 0.234, 2.80922, -.29, 9.87]:
        sino, angles = gauss_sino_3d_tilted(tilt_plane=angz, A=21)
        axis = np.dot(np.array([[np.cos(angz), -np.sin(angz), 0],
                                [np.sin(angz), np.cos(angz), 0],
                                [0, 0, 1]]), [0, 1, 0])
        f = odt.backpropagate_3d_tilted(sino, angles, padval="edge",
                                        tilted_axis=axis,
                                        padding=(False, False), **p)
        results.append(cutout(f).flatten().view(float))
    for ii in range(len(results)):
        assert np.allclose(results[ii], results[ii - 1], atol=.2, rtol=.2)


def test_multibatch_kahan(odt, monkeypatch):
    """A workspace too small for all angles forces several batches; the
    compensation carried across launches keeps the result unchanged."""
    from odtbrain_gb300 import _alg3d
    sino, angles = ellipsoid_phantom_sinogram(48, 40, seed=4,
                                              count_range=(2, 4),
                                              semi_range=(4, 12))
    kw = dict(res=3.0, nm=1.333, dtype=np.float32)
    one = odt.backpropagate_3d(sino, angles, **kw)
    monkeypatch.setattr(_alg3d, "_WS_DEFAULT", 8 << 20)
    _alg3d._PLAN_CACHE.clear()
    many = odt.backpropagate_3d(sino, angles, **kw)
    _alg3d._PLAN_CACHE.clear()
    ref = O.backpropagate_3d(sino, angles, res=3.0, nm=1.333)
    assert_close(many, ref, what="multibatch")
    assert_close(one, ref, what="single batch")


def test_single_row_multibatch(odt, cuda_ready):
    """A single-row plan (the fused column + row stage) over several angle
    batches: the compensation carried across the resampling launches and
    the per-batch z-boundary rows keep the result unchanged."""
    import torch
    from odtbrain_gb300._alg3d import Backprop3D
    rng = np.random.default_rng(21)
    A, nx = 40, 64
    shape = (A, 1, nx)
    sino = np.exp(1j * rng.normal(0, .4, shape) + rng.normal(0, .05, shape))
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    ref = O.backpropagate_3d(sino, angles, res=3.0, nm=1.333,
                             padding=(False, False))
    d = torch.from_numpy(sino).to(cuda_ready)
    one = Backprop3D(shape, angles, 3.0, 1.333, padding=(False, False),
                     input_dtype="complex128", device=cuda_ready)
    many = Backprop3D(shape, angles, 3.0, 1.333, padding=(False, False),
                      input_dtype="complex128", device=cuda_ready,
                      workspace_limit=256 << 10)
    # five launches per batch: row spectra, boundary columns, fused
    # column + row stage, geometry setup, resampling
    assert one.launches_per_call == 5 and many.launches_per_call > 10
    assert_close(one(d).cpu().numpy(), ref, what="single batch")
    assert_close(many(d).cpu().numpy(), ref, what="multibatch")


def test_torch_tensors_in_and_out(odt):
    import torch
    sino, angles = gauss_sino_3d()
    p = parameter_sets(1)[0]
    ref = odt.backpropagate_3d(sino, angles, dtype=np.float32, **p)
    t = torch.from_numpy(sino.astype(np.complex64)).cuda()
    out = odt.backpropagate_3d(t, torch.from_numpy(angles), dtype=np.float32,
                               **p)
    assert isinstance(out, torch.Tensor) and out.is_cuda
    assert out.dtype == torch.complex64
    assert np.allclose(out.cpu().numpy(), ref, rtol=0,
                       atol=1e-6 * np.abs(ref).max())


def test_c2_shape_subset_vs_oracle(odt):
    """256^2 -> 512^2 padded, 256^3 volume (the benchmark's plane and volume
    size) with 3 angles; the oracle runs on the host cores."""
    sino, angles = ellipsoid_phantom_sinogram(
        256, 3, seed=11, count_range=(3, 12), semi_range=(8, 60),
        angles=np.array([0.3, 1.9, 4.4]))
    kw = dict(res=3.0, nm=1.333)
    got = odt.backpropagate_3d(sino.astype(np.complex64), angles,
                               dtype=np.float32, **kw)
    ref = O.backpropagate_3d(sino, angles, fft_workers=-1, **kw)
    assert_close(got, ref, what="256^3")


def test_c3_shape_subset_vs_oracle(odt):
    """Tilted axis 0.2 rad toward z, 200^2 -> 512^2, 200^3 volume, 2
    angles."""
    ax = (0, np.cos(0.2), np.sin(0.2))
    sino, angles = ellipsoid_phantom_sinogram(
        200, 2, seed=12, count_range=(3, 12), semi_range=(8, 50), axis=ax,
        angles=np.array([0.0, 2.5]))
    # two angles give 0/0 angle weights (as in the reference): weights off
    kw = dict(res=3.0, nm=1.333, tilted_axis=ax, weight_angles=False)
    got = odt.backpropagate_3d_tilted(sino.astype(np.complex64), angles,
                                      dtype=np.float32, **kw)
    ref = O.backpropagate_3d_tilted(sino, angles, fft_workers=-1, **kw)
    assert_close(got, ref, what="200^3 tilted")


def test_full_c1_vs_reference_and_oracle(odt):
    """The whole 60-angle, 64x64 -> 64^3 workload (ellipsoid phantom,
    padfac 1.75 -> 128^2 FFTs, order 2, angle weights on, complex output):
    the GPU result against the unmodified reference's output (fixture) and
    against the FP64 oracle run here, rel-L2 <= 1e-5 and max <= 1e-5 of
    the largest magnitude.  The fixture stores float32 parts (rounding
    ~3e-8), well inside the bound."""
    sino, angles, kw, ref = reference_c1()
    got = odt.backpropagate_3d(sino, angles, dtype=np.float64, **kw)
    assert got.dtype == np.complex128
    assert_close(got, ref, what="C1 vs reference")
    kw_o = dict(kw)
    kw_o.pop("onlyreal")
    oracle = O.backpropagate_3d(sino, angles, **kw_o)
    assert_close(got, oracle, what="C1 vs oracle")


def test_device_check_status_raises(odt, cuda_ready):
    """A kernel's own check records bits in the plan's status word; the
    next status read turns them into ODT_ERR_DEVICE_CHECK and a Python
    exception, clears the word, and the plan keeps working.  The bits are
    set by the host (odt_debug_inject_status), so no kernel is made to
    fail."""
    import ctypes
    import torch
    from odtbrain_gb300 import _native
    from odtbrain_gb300._alg3d import Backprop3D
    sino, angles = ellipsoid_phantom_sinogram(32, 12, seed=5,
                                              count_range=(1, 3),
                                              semi_range=(3, 8))
    rec = Backprop3D(sino.shape, angles, 3.0, 1.333,
                     input_dtype="complex128", device=cuda_ready)
    d = torch.from_numpy(sino).to(cuda_ready)
    first = rec(d).cpu().numpy()
    stream = torch.cuda.current_stream(cuda_ready)
    handle = ctypes.c_void_p(stream.cuda_stream)
    rec.plan.inject_status(1, handle)  # DEVCHK_BOX_OVERFLOW
    with pytest.raises(_native.OdtError, match="bits 0x1") as info:
        rec.check()
    assert info.value.status == _native.ODT_ERR_DEVICE_CHECK
    rec.check()  # cleared by the read
    # the same bits arriving between a launch and the status read of a call
    rec.plan.inject_status(2, handle)  # DEVCHK_BAD_CONFIG
    with pytest.raises(_native.OdtError, match="bits 0x2"):
        rec(d)
    again = rec(d).cpu().numpy()
    np.testing.assert_array_equal(first, again)
    ref = O.backpropagate_3d(sino, angles, res=3.0, nm=1.333)
    assert_close(again, ref, what="after a device check")


# The full benchmark configurations (their seeded workloads, every angle):
# the benchmark spec states its rel-L2 target for these sizes.
FULL_CONFIGS = {
    "c2": dict(n=256, A=200, seed=2024, count_range=(3, 12),
               semi_range=(8, 60), axis=None),
    "c3": dict(n=200, A=220, seed=2025, count_range=(3, 12),
               semi_range=(8, 50),
               axis=(0.0, float(np.cos(0.2)), float(np.sin(0.2)))),
}


@pytest.mark.parametrize("cfg", ["c2", "c3"])
def test_full_config_vs_oracle(odt, cfg):
    """The 200-angle 256^2 -> 256^3 workload (y axis) and the 220-angle
    200^2 -> 200^3 workload (axis tilted 0.2 rad toward z), complex64 input,
    angle weights on, padfac 1.75 (512^2 FFTs), order 2: every angle against
    the FP64 oracle (about a minute of host time each), rel-L2 <= 1e-5 and
    max <= 1e-5 of the largest magnitude."""
    c = FULL_CONFIGS[cfg]
    ax = c["axis"]
    sino, angles = ellipsoid_phantom_sinogram(
        c["n"], c["A"], seed=c["seed"], count_range=c["count_range"],
        semi_range=c["semi_range"], axis=ax or (0, 1, 0))
    sino = sino.astype(np.complex64)
    kw = dict(res=3.0, nm=1.333, padfac=1.75, intp_order=2)
    if ax is None:
        got = odt.backpropagate_3d(sino, angles, dtype=np.float32, **kw)
        ref = O.backpropagate_3d(sino.astype(np.complex128), angles,
                                 fft_workers=-1, **kw)
    else:
        got = odt.backpropagate_3d_tilted(sino, angles, dtype=np.float32,
                                          tilted_axis=ax, **kw)
        ref = O.backpropagate_3d_tilted(sino.astype(np.complex128), angles,
                                        tilted_axis=ax, fft_workers=-1, **kw)
    assert_close(got, ref, what="%s full" % cfg)


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5])
@pytest.mark.parametrize("kind", ["y", "tilted"])
def test_pow2_rows_any_crop(odt, order, kind):
    """Rectangular 60x100 planes padded to 128x256: the power-of-two row
    stage with a crop that is not the centred half (pad 78 of 256), every
    spline order, both geometries, against the FP64 oracle."""
    rng = np.random.default_rng(100 + order + 10 * (kind == "y"))
    A, ny, nx = 4, 60, 100
    sino = (1 + rng.normal(0, .05, (A, ny, nx))
            + 1j * rng.normal(0, .3, (A, ny, nx)))
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    kw = dict(res=3.0, nm=1.333, intp_order=order, padval="edge",
              weight_angles=False)
    if kind == "y":
        ref = O.backpropagate_3d(sino, angles, fft_workers=-1, **kw)
        got = odt.backpropagate_3d(sino, angles, **kw)
    else:
        ax = (0.1, np.cos(0.3), np.sin(0.3))
        ref = O.backpropagate_3d_tilted(sino, angles, tilted_axis=ax,
                                        fft_workers=-1, **kw)
        got = odt.backpropagate_3d_tilted(sino, angles, tilted_axis=ax, **kw)
    assert_close(got, ref, what="order %d %s 60x100" % (order, kind))


@pytest.mark.parametrize("order", [4, 5])
def test_high_orders_full_planes(odt, order):
    """Quartic and quintic splines (two prefilter poles) on 256^2 -> 512^2
    planes, the centred-half crop of the benchmark's shapes, 3 angles, both
    geometries, against the FP64 oracle."""
    sino, angles = ellipsoid_phantom_sinogram(
        256, 3, seed=13 + order, count_range=(3, 8), semi_range=(8, 60),
        angles=np.array([0.4, 2.1, 4.0]))
    kw = dict(res=3.0, nm=1.333, intp_order=order, weight_angles=False)
    got = odt.backpropagate_3d(sino.astype(np.complex64), angles,
                               dtype=np.float32, **kw)
    ref = O.backpropagate_3d(sino, angles, fft_workers=-1, **kw)
    assert_close(got, ref, what="order %d, 256^3" % order)
    ax = (0, np.cos(0.2), np.sin(0.2))
    got = odt.backpropagate_3d_tilted(sino.astype(np.complex64), angles,
                                      dtype=np.float32, tilted_axis=ax, **kw)
    ref = O.backpropagate_3d_tilted(sino, angles, tilted_axis=ax,
                                    fft_workers=-1, **kw)
    assert_close(got, ref, what="order %d, tilted 256^3" % order)
