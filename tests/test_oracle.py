"""CPU tests that pin the FP64 oracle before it is trusted as the checker.

* against the reference's own golden vectors (tests/data/alg3d_bpp__*.zip of
  the reference, re-saved in tests/golden/reference_zips.npz);
* against outputs of the unmodified reference (tests/golden/
  reference_cases.npz, made by tests/golden/make_golden.py);
* the C spline resampler against the installed scipy.ndimage, whose
  rotate/affine_transform the reference calls
  (odtbrain/_alg3d_bpp.py:73-81, odtbrain/_alg3d_bppt.py:931-944).
"""
import numpy as np
import pytest
import scipy.ndimage as ndi

from conftest import reference_c1, reference_cases
from oracle import odt_oracle as O
from sino_gen import cutout, parameter_sets, gauss_sino_3d


def test_golden_backprop_phase(golden):
    """test_alg3d_bpp.py:30-42 against its zip."""
    sino, angles = gauss_sino_3d()
    r = [cutout(O.backpropagate_3d(sino, angles, padval=0, **p))
         for p in parameter_sets(2)]
    data = np.array(r).flatten().view(float)
    ref = golden["reference_zips"]["test_3d_backprop_phase"]
    assert np.allclose(data, ref)
    assert np.abs(data - ref).max() < 1e-9


def test_golden_backprop_nopadreal(golden):
    """test_alg3d_bpp.py:45-62 against its zip."""
    sino, angles = gauss_sino_3d()
    r = [cutout(O.backpropagate_3d(sino, angles, padding=(False, False),
                                   onlyreal=True, **p))
         for p in parameter_sets(2)]
    data = np.array(r).flatten().view(float)
    ref = golden["reference_zips"]["test_3d_backprop_nopadreal"]
    assert np.allclose(data, ref)
    assert np.abs(data - ref).max() < 1e-9


def test_golden_mprotate(golden):
    """test_alg3d_bpp.py:116-134: first 10 y-planes of a 20^3 arange volume
    rotated by -2 degrees at order 2, the rest untouched."""
    ln2 = 20
    arr = np.arange(ln2 ** 3, dtype=float).reshape(ln2, ln2, ln2)
    out = arr.copy()
    out[:, :10, :] = O.rotate_planes_y(arr[:, :10, :], -2, 2)
    ref = golden["reference_zips"]["test_3d_mprotate"]
    assert np.allclose(out.flatten(), ref)


def test_reference_cases(golden):
    """Oracle == unmodified reference on every stored case (FP64)."""
    n = 0
    for name, sino, angles, kw, out in reference_cases(golden):
        fn = (O.backpropagate_3d_tilted if name.startswith("bppt")
              else O.backpropagate_3d)
        got = fn(sino, angles, **kw)
        scale = np.abs(out).max()
        assert got.shape == out.shape, name
        assert np.abs(got - out).max() <= 1e-11 * scale, name
        n += 1
    assert n >= 8


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5])
def test_rotate_matches_scipy(order):
    rng = np.random.default_rng(order)
    for trial in range(6):
        nz, ny, nx = rng.integers(2, 19), rng.integers(1, 4), \
            rng.integers(2, 19)
        if trial == 0:
            nz = nx = 16
        vol = rng.standard_normal((nz, ny, nx))
        ang = [0.0, 90.0, -180.0, 33.3, -271.0,
               rng.uniform(-360, 360)][trial]
        ref = ndi.rotate(vol, ang, axes=(0, 2), reshape=False, order=order,
                         mode="constant", cval=0)
        got = O.rotate_planes_y(vol, ang, order)
        assert np.abs(got - ref).max() < 1e-11 * max(1, np.abs(ref).max())
        assert np.array_equal(got == 0, ref == 0)


@pytest.mark.parametrize("order", [0, 1, 2, 3, 4, 5])
def test_affine3d_matches_scipy(order):
    from scipy.spatial.transform import Rotation
    rng = np.random.default_rng(10 + order)
    for trial in range(3):
        shape = tuple(int(v) for v in rng.integers(3, 14, 3))
        vol = rng.standard_normal(shape)
        mat = Rotation.from_rotvec(rng.standard_normal(3)).as_matrix()
        c = 0.5 * np.array(shape) - .5
        off = c - mat @ c
        ref = ndi.affine_transform(vol, mat, offset=off, order=order,
                                   mode="constant", cval=0)
        got = O.affine_transform_3d(vol, mat, off, order)
        assert np.abs(got - ref).max() < 1e-11 * max(1, np.abs(ref).max())


def test_prefilter_matches_scipy():
    rng = np.random.default_rng(5)
    for order in (2, 3, 4, 5):
        for n in (2, 3, 5, 17, 64):
            line = rng.standard_normal(n)
            ref = ndi.spline_filter1d(line, order, mode="mirror")
            got = O.spline_filter_line(line, order)
            assert np.abs(got - ref).max() < 1e-12 * max(1, abs(ref).max())


def test_boundary_exactness_scipy_order():
    """Coordinates evaluated ((off + m0*o0) + m1*o1) reproduce scipy's
    out-of-domain decisions at every edge voxel, including angles whose
    cosine is not exactly representable."""
    rng = np.random.default_rng(1)
    for n in (22, 64, 63):
        vol = rng.standard_normal((n, 1, n)) + 5
        for deg in np.rad2deg(np.linspace(0, 2 * np.pi, 60, endpoint=False)):
            ref = ndi.rotate(vol, -deg, axes=(0, 2), reshape=False, order=1,
                             mode="constant", cval=0)
            got = O.rotate_planes_y(vol, -deg, 1)
            assert np.array_equal(got == 0, ref == 0)


def test_angle_weights_known_answers():
    """test_util.py:6-32 of the reference."""
    res = O.compute_angle_weights_1d(np.linspace(0, np.pi, 18,
                                                 endpoint=False))
    assert np.allclose(res, 1, rtol=0, atol=1e-14)
    angles = np.linspace(0, np.pi, 18, endpoint=True)
    res = O.compute_angle_weights_1d(angles)
    assert np.allclose(np.mean(res), 1, rtol=0, atol=1e-14)
    assert np.allclose(res[1:-1], 18 / 17, rtol=0, atol=1e-14)
    assert np.allclose(res[[0, -1]], 18 / 17 / 2, rtol=0, atol=1e-14)
    a0 = np.linspace(0, np.pi, 14, endpoint=False)
    a2 = np.concatenate((np.ones(4) * np.roll(a0, -3)[0], np.roll(a0, -3)))
    res = O.compute_angle_weights_1d(np.roll(a2, 3))
    assert np.allclose(np.mean(res), 1, rtol=0, atol=1e-14)
    assert np.allclose(res[:3], 18 / 14, rtol=0, atol=1e-14)
    assert np.allclose(res[3 + 4 + 1:], 18 / 14, rtol=0, atol=1e-14)
    assert np.allclose(res[3:8], 18 / 14 / 5, rtol=0, atol=1e-14)


def test_oracle_weights_match_reference(golden):
    g = golden["reference_geometry"]
    for k in [k for k in g if k.startswith("weights_") and
              k.endswith("__angles")]:
        stem = k[:-len("__angles")]
        got = O.compute_angle_weights_1d(g[k])
        assert np.array_equal(got, g[stem + "__w"]), stem


@pytest.mark.parametrize("order", [1, 2, 3])
def test_dense_model_matches_oracle(order):
    """The dense FP64 torch model (used to check the adjoint with autograd)
    reproduces the oracle."""
    import torch
    from dense_model import DenseBackprop
    rng = np.random.default_rng(40 + order)
    A, n = 5, 12
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    sino = rng.normal(0, .3, (A, n, n)) + 1j * rng.normal(0, 1, (A, n, n))
    model = DenseBackprop(angles, n, n, 3.0, 1.333, order=order)
    got = model(torch.from_numpy(sino)).numpy()
    ref = O.backpropagate_3d(sino, angles, 3.0, 1.333, intp_order=order)
    assert np.abs(got - ref).max() <= 1e-12 * np.abs(ref).max()


def test_oracle_full_c1_matches_reference():
    """The whole 60-angle, 64x64 -> 64^3 workload (128^2 FFTs, order 2,
    weights on) against the unmodified reference's output for it; the
    fixture holds float32 real/imaginary parts, so the bound is FP32
    storage rounding."""
    sino, angles, kw, ref = reference_c1()
    kw = dict(kw)
    assert kw.pop("onlyreal") is False
    got = O.backpropagate_3d(sino, angles, **kw)
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    mx = np.abs(got - ref).max() / np.abs(ref).max()
    assert rel < 2e-7 and mx < 2e-7, (rel, mx)
