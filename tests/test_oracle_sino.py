"""CPU tests of the sinogram-preparation oracle (oracle/unwrap_oracle.py)
against the reference's golden vectors and reference-made fixtures, and of
the host helpers of odtbrain_gb300._prepare_sino.

Mirrors the reference's tests/test_processing.py:78-148."""
import json
import os

import numpy as np
import pytest

from oracle import unwrap_oracle as uo
from odtbrain_gb300 import _prepare_sino

TWOPI = 2 * np.pi
GOLDEN = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


@pytest.fixture(scope="module")
def sino_fix():
    with np.load(os.path.join(GOLDEN, "reference_sino.npz")) as z:
        return {k: z[k] for k in z.files}


def processing_sino(rytov=False):
    """tests/test_processing.py:24-32 of the reference."""
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


def fixture_cases(fx):
    names = sorted({k.split("__")[0] for k in fx if "__" in k})
    for n in names:
        yield (n, fx[n + "__sino"], fx.get(n + "__u0"),
               json.loads(str(fx[n + "__kw"])), fx[n + "__out"])


def test_oracle_sino_rytov_golden(sino_fix):
    ryt = uo.sinogram_as_rytov(processing_sino(rytov=True))
    if ryt.imag.min() > TWOPI:
        ryt.imag -= TWOPI
    assert np.allclose(np.array(ryt).flatten().view(float),
                       sino_fix["zip_test_sino_rytov"])
    s = processing_sino(rytov=True)
    for two, three in ((s[:, :, 0], ryt[:, :, 0]), (s[:, 0, :], ryt[:, 0, :])):
        d = uo.sinogram_as_rytov(two) - three
        assert np.allclose(0, d.real, atol=1e-6)
        assert np.allclose(0, negative_modulo_rest(d.imag, TWOPI), atol=1e-6)


def test_oracle_sino_radon_golden(sino_fix):
    rad = uo.sinogram_as_radon(processing_sino())
    if rad.min() > TWOPI:
        rad -= TWOPI
    assert np.allclose(rad.ravel(), sino_fix["zip_test_sino_radon"])


def test_oracle_matches_reference_runs(sino_fix):
    n = 0
    for name, sino, u0, kw, out in fixture_cases(sino_fix):
        args = {} if u0 is None else {"u0": u0}
        if kw["kind"] == "rytov":
            got = uo.sinogram_as_rytov(sino, align=kw["align"], **args)
        else:
            got = uo.sinogram_as_radon(sino, align=kw["align"])
        assert got.dtype == out.dtype, name
        tol = 1e-5 if out.dtype in (np.complex64, np.float32) else 1e-12
        np.testing.assert_allclose(got, out, rtol=tol, atol=tol, err_msg=name)
        n += 1
    assert n == 13


def test_divmod_neg_known_answers():
    """tests/test_processing.py:140-148 of the reference, for the oracle and
    the package's host helper."""
    for fn in (uo.divmod_neg, _prepare_sino.divmod_neg):
        assert np.allclose(fn(0, TWOPI), (0, 0))
        assert np.allclose(fn(-1e-17, TWOPI), (0, 0))
        assert np.allclose(fn(1e-17, TWOPI), (0, 0))
        assert np.allclose(fn(-.1, TWOPI), (0, -.1))
        assert np.allclose(fn(.1, TWOPI), (0, .1))
        assert np.allclose(fn(3 * np.pi, TWOPI), (1, np.pi))
        assert np.allclose(fn(-.99 * np.pi, TWOPI), (0, -.99 * np.pi))
        assert np.allclose(fn(-1.01 * np.pi, TWOPI), (-1, .99 * np.pi))


def test_oracle_unwrap_recovers_smooth_phase():
    y, x = np.mgrid[:31, :27]
    true = 14 * np.exp(-((y - 14.0) ** 2 + (x - 12.0) ** 2) / 60.0)
    w = np.angle(np.exp(1j * true))
    for anchor in ("head", "first_edge"):
        u = uo.unwrap_2d(w, anchor=anchor)
        k = np.round((u - true) / TWOPI)
        assert len(np.unique(k)) == 1
        assert np.allclose(u - TWOPI * k, true, atol=1e-12)


def test_oracle_anchor_keeps_wrapped_value():
    rng = np.random.default_rng(3)
    w = np.angle(np.exp(1j * rng.normal(0, 2.5, (9, 13))))
    u = uo.unwrap_2d(w, anchor="first_edge")
    p = uo.first_edge_pixel(w)
    assert u.ravel()[p] == w.ravel()[p]
    u2, head = uo.unwrap_2d(w, return_head=True)
    assert u2.ravel()[head] == w.ravel()[head]
    k = np.round((u - w) / TWOPI)
    assert np.allclose(u, w + TWOPI * k)


def test_border_noise_range_and_determinism():
    v = uo.border_noise(47, np.arange(1000))
    assert v.min() >= 0 and v.max() < 2 ** 31
    assert np.array_equal(v, uo.border_noise(47, np.arange(1000)))
    assert not np.array_equal(v, uo.border_noise(48, np.arange(1000)))


def test_complex_dtype_promotion():
    cd = _prepare_sino._complex_dtype
    assert cd(np.result_type(np.complex64, 1)) == np.complex64
    assert cd(np.result_type(np.complex64, np.complex128)) == np.complex128
    assert cd(np.result_type(np.float32, 2.0)) == np.complex64
    assert cd(np.result_type(np.int64, 1)) == np.complex128
