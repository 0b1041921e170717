"""The spline prefilter folded into the FFT stages, checked in FP64 against
scipy.ndimage (CPU, no GPU).

scipy prefilters each resampled axis of the cropped slab with mirror
boundaries before the B-spline interpolation
(odtbrain/_alg3d_bpp.py:79 -> scipy.ndimage.rotate -> spline_filter1d).
The filter stages instead divide the padded spectrum by the sampled
B-spline's transfer function B(k) and add, per cropped line of n samples,
the homogeneous terms sum_i A_i z_i^k + B_i z_i^(n-1-k) of the pole(s) z_i,
with (A, B) from the mirror conditions c[m] = c[-m], c[n-1-m] = c[n-1+m]
(m = 1..poles) evaluated on the line's samples around the crop.  This test
restates that construction in NumPy (one pole for orders 2-3, two for 4-5)
and compares it with scipy's own prefilter of the cropped line.
"""
import math

import numpy as np
import pytest
from scipy import ndimage


def bspline_samples(order):
    """Centred B-spline of `order` at the integers -order//2 .. order//2."""
    half = order // 2
    out = []
    for m in range(-half, half + 1):
        x = m + (order + 1) / 2.0
        v = sum((-1) ** j * math.comb(order + 1, j) * max(x - j, 0.0) ** order
                for j in range(order + 2)) / math.factorial(order)
        out.append(v)
    return np.array(out)


def poles(order):
    """Roots of the B-spline's Laurent polynomial inside the unit circle."""
    b = bspline_samples(order)
    r = np.roots(b[::-1])
    return np.sort(np.real(r[np.abs(r) < 1]))


def folded_prefilter(spec, pad, n, order):
    """Prefiltered coefficients of samples pad..pad+n-1 of ifft(spec)."""
    L = spec.size
    b = bspline_samples(order)
    half = order // 2
    k = 2 * np.pi * np.fft.fftfreq(L)
    bhat = sum(b[i] * np.cos(k * (i - half)) for i in range(b.size))
    u = np.fft.ifft(spec / bhat)  # particular solution on the periodic line
    z = poles(order)
    np_ = z.size

    def uu(i):  # sample i relative to pad (periodic)
        return u[(pad + i) % L]

    # unknowns A_1..A_np, B_1..B_np; rows: left then right mirror conditions
    M = np.zeros((2 * np_, 2 * np_))
    d = np.zeros(2 * np_, dtype=complex)
    for m in range(1, np_ + 1):
        d[m - 1] = uu(m) - uu(-m)
        d[np_ + m - 1] = uu(n - 1 - m) - uu(n - 1 + m)
        for i, zi in enumerate(z):
            M[m - 1, i] = zi ** m - zi ** (-m)
            M[m - 1, np_ + i] = zi ** (n - 1 - m) - zi ** (n - 1 + m)
            M[np_ + m - 1, i] = zi ** (n - 1 - m) - zi ** (n - 1 + m)
            M[np_ + m - 1, np_ + i] = zi ** m - zi ** (-m)
    coef = np.linalg.solve(M, -d)
    kk = np.arange(n)
    c = u[(pad + kk) % L].copy()
    for i, zi in enumerate(z):
        c += coef[i] * zi ** kk + coef[np_ + i] * zi ** (n - 1 - kk)
    return c


@pytest.mark.parametrize("order", [2, 3, 4, 5])
@pytest.mark.parametrize("L,pad,n", [(512, 128, 256), (512, 156, 200),
                                     (128, 32, 64), (256, 78, 100)])
def test_folded_prefilter_matches_scipy(order, L, pad, n):
    rng = np.random.default_rng(order * 1000 + L + pad)
    spec = rng.normal(size=L) + 1j * rng.normal(size=L)
    x = np.fft.ifft(spec)[pad:pad + n]
    ref = (ndimage.spline_filter1d(x.real, order=order, mode="mirror")
           + 1j * ndimage.spline_filter1d(x.imag, order=order, mode="mirror"))
    got = folded_prefilter(spec, pad, n, order)
    err = np.abs(got - ref).max() / np.abs(ref).max()
    assert err < 1e-12, (order, L, pad, n, err)


def test_pole_values():
    """The poles of orders 2-5 (Unser's B-spline filter design)."""
    assert np.allclose(poles(2), [np.sqrt(8.0) - 3.0])
    assert np.allclose(poles(3), [np.sqrt(3.0) - 2.0])
    assert poles(4).size == 2 and poles(5).size == 2
    assert np.all(np.abs(poles(4)) < 1) and np.all(poles(5) < 0)
