"""CPU tests of the apple-core oracle (oracle/apple_oracle.py) against the
reference's golden vector and reference-made fixtures; mirrors the
reference's tests/test_apple.py."""
import json
import os

import numpy as np
import pytest

import apple_helper_cases
from oracle import apple_oracle as ao
from oracle import odt_oracle, unwrap_oracle
from sino_gen import cutout, gauss_sino_3d

GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def apple_fix():
    with np.load(os.path.join(GOLDEN, "reference_apple.npz")) as z:
        return {k: z[k] for k in z.files}


@pytest.fixture(scope="module")
def zips():
    with np.load(os.path.join(GOLDEN, "reference_sino.npz")) as z:
        return {k: z[k] for k in z.files if k.startswith("zip_")}


def apple_cases(fx):
    names = sorted({k.split("__")[0] for k in fx if "__" in k})
    for n in names:
        kw = json.loads(str(fx[n + "__kw"]))
        if n + "__mask" in fx:
            kw["mask"] = fx[n + "__mask"]
        yield n, fx["vol_" + str(fx[n + "__vol"])], kw, fx[n + "__out"]


def golden_input():
    """tests/test_apple.py:48-61 of the reference, up to apple.correct."""
    sino, angles = gauss_sino_3d(A=9, Nx=10, Ny=10)
    sryt = unwrap_oracle.sinogram_as_rytov(sino, u0=1, align=False)
    return odt_oracle.backpropagate_3d(sryt, angles, res=2.1, nm=1.333,
                                       lD=0, padval=0)


def test_oracle_correct_reproduce_golden(zips):
    fc = ao.correct(f=golden_input(), res=2.1, nm=1.333,
                    enforce_envelope=.95, max_iter=100, min_diff=0.01)
    fo = np.array(cutout(fc), dtype=np.complex128)
    assert np.allclose(fo.flatten().view(float),
                       zips["zip_test_correct_reproduce"], atol=2.E-6)


def test_oracle_matches_reference_runs(apple_fix):
    n = 0
    for name, f, kw, out in apple_cases(apple_fix):
        got = ao.correct(f=f.copy(), **kw)
        assert got.dtype == np.complex64
        np.testing.assert_allclose(got, out, rtol=0, atol=1e-6,
                                   err_msg=name)
        n += 1
    assert n == 9


def test_apple_core_shape_error():
    """tests/test_apple.py:16-24 of the reference."""
    with pytest.raises(ValueError):
        ao.apple_core_3d(shape=(10, 10, 5), res=.1, nm=1)


def test_envelope_non_cubic_shape():
    """tests/test_apple.py:90-97 of the reference."""
    shape = (60, 50, 60)
    core = ao.apple_core_3d(shape=shape, res=.1, nm=1)
    assert ao.envelope_gauss(ftdata=np.ones(shape), core=core).shape == shape


def test_enforce_envelope_range():
    """tests/test_apple.py:72-87 of the reference."""
    with pytest.raises(ValueError):
        ao.correct(np.zeros((4, 4, 4)), res=2.1, nm=1.333,
                   enforce_envelope=1.05)


@pytest.fixture(scope="module")
def helper_fix():
    return apple_helper_cases.load()


def test_oracle_constraints_match_reference(helper_fix):
    """constraint_nn / constraint_sh (apple.py:56-110) on float32, float64,
    complex64 and complex128 data, with and without mask and shell: the
    oracle reproduces the reference's in-place results bit for bit."""
    n = 0
    for name, fn, data, kw, ref in apple_helper_cases.constraint_cases(helper_fix):
        getattr(ao, fn)(data, **kw)
        assert data.dtype == ref.dtype
        np.testing.assert_array_equal(data, ref, err_msg=name)
        n += 1
    assert n == 9


def test_oracle_envelope_matches_reference(helper_fix):
    """envelope_gauss (apple.py:289-350), cubic and both non-cubic padding
    directions, complex64 and complex128 spectra: bit for bit."""
    n = 0
    for name, ft, core, ref in apple_helper_cases.envelope_cases(helper_fix):
        got = ao.envelope_gauss(ft.copy(), core)
        assert got.dtype == ref.dtype
        np.testing.assert_array_equal(got, ref, err_msg=name)
        n += 1
    assert n == 5
