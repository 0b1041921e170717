"""GPU tests of the 2D backpropagation and of the refractive-index
conversions (drop-ins for odtbrain.backpropagate_2d, odt_to_ri,
opt_to_ri): against the reference's golden vectors and reference-made
fixtures, the FP64 oracle, and the reference's property tests
(tests/test_alg2d_bpp.py, tests/test_processing.py)."""
import multiprocessing as mp

import numpy as np
import pytest

from oracle import odt_oracle as O
from sino_gen import cutout, gauss_sino_2d, parameter_sets

pytestmark = pytest.mark.gpu
REL = 1e-5


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - b) / np.linalg.norm(b)


def test_2d_reference_cases(cuda_ready, golden):
    import odtbrain_gb300 as odt
    from conftest import reference_cases
    for n, sino, angles, kw, ref in reference_cases(golden, two_d=True):
        out = odt.backpropagate_2d(sino, angles, **kw)
        assert out.shape == ref.shape and out.dtype == ref.dtype, n
        assert _rel(out, ref) < REL, (n, _rel(out, ref))
        assert np.abs(out - ref).max() <= 2 * REL * np.abs(ref).max(), n


@pytest.mark.parametrize("name,ampl", [("test_2d_backprop_phase", (1., 1.)),
                                       ("test_2d_backprop_full", (.9, 1.1))])
def test_2d_reference_zips(cuda_ready, golden, name, ampl):
    import odtbrain_gb300 as odt
    sino, angles = gauss_sino_2d(ampl_range=ampl)
    r = [cutout(odt.backpropagate_2d(sino, angles, **p))
         for p in parameter_sets(2)]
    got = np.array(r).flatten().view(float)
    assert _rel(got, golden["reference_zips"][name]) < REL


def test_2d_real_is_real_part(cuda_ready):
    import odtbrain_gb300 as odt
    sino, angles = gauss_sino_2d()
    for p in parameter_sets(2):
        f = odt.backpropagate_2d(sino, angles, padval=0, **p)
        g = odt.backpropagate_2d(sino, angles, padval=0, onlyreal=True, **p)
        assert g.dtype == np.float64
        assert np.allclose(f.real, g, rtol=0, atol=1e-6 * np.abs(f).max())


def test_2d_against_oracle_larger(cuda_ready):
    import odtbrain_gb300 as odt
    rng = np.random.default_rng(4)
    A, N = 60, 96
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    sino = (rng.normal(0, .05, (A, N)) + 1j * rng.normal(0, 1, (A, N)))
    for kw in (dict(padval=0), dict(padval=None), dict(padding=False),
               dict(padval=0.5, lD=3.0, weight_angles=False)):
        got = odt.backpropagate_2d(sino, angles, 3.2, 1.333, **kw)
        ref = O.backpropagate_2d(sino, angles, 3.2, 1.333, **kw)
        assert _rel(got, ref) < REL, kw


@pytest.mark.parametrize("N,A", [(1000, 3), (500, 7), (21, 9)])
def test_2d_line_lengths(cuda_ready, N, A):
    """Padded line lengths 4096, 2048 and 64: every thread layout of the
    fused single-row stage (one 512-thread line per group, one 256-thread
    line, 32 lines of 8 threads) against the oracle."""
    import odtbrain_gb300 as odt
    rng = np.random.default_rng(N)
    angles = np.sort(rng.uniform(0, 2 * np.pi, A))
    x = np.linspace(-1, 1, N)
    sino = (np.exp(-x ** 2 / 0.1)[None, :] * rng.uniform(0.5, 2, (A, 1))
            + 0.02 * rng.normal(size=(A, N))) * 1j
    got = odt.backpropagate_2d(sino, angles, 3.0, 1.333)
    ref = O.backpropagate_2d(sino, angles, 3.0, 1.333)
    assert _rel(got, ref) < REL


def test_2d_torch_and_counters(cuda_ready):
    import torch
    import odtbrain_gb300 as odt
    sino, angles = gauss_sino_2d()
    count, max_count = mp.Value("i", 0), mp.Value("i", 0)
    ref = odt.backpropagate_2d(sino, angles, 2.1, 1.333, count=count,
                               max_count=max_count)
    assert max_count.value == len(angles) + 2
    assert count.value == max_count.value
    t = odt.backpropagate_2d(torch.tensor(sino, device=cuda_ready),
                             torch.tensor(angles), 2.1, 1.333)
    assert t.is_cuda and t.dtype == torch.complex128
    assert np.allclose(t.cpu().numpy(), ref)


def test_2d_errors(cuda_ready):
    import odtbrain_gb300 as odt
    sino, angles = gauss_sino_2d()
    with pytest.raises(AssertionError):
        odt.backpropagate_2d(sino[None], angles, 2.1, 1.333)
    with pytest.raises(AssertionError):
        odt.backpropagate_2d(sino[:-1], angles, 2.1, 1.333)
    with pytest.raises(TypeError):
        odt.backpropagate_2d(sino, angles, 2.1, 1.333, coords=np.zeros(3))


def _ri_data():
    ln = 10
    f = np.arange(ln ** 3).reshape(ln, ln, ln)
    return f + np.linspace(1, 2, ln), 7, 1.34


def test_ri_reference_zips_and_2d(cuda_ready, golden):
    import odtbrain_gb300 as odt
    f, res, nm = _ri_data()
    z = golden["reference_zips"]
    ri = odt.odt_to_ri(f=f, res=res, nm=nm)
    assert ri.dtype == np.float64
    assert np.allclose(np.array(ri).flatten().view(float), z["test_odt_to_ri"])
    assert np.allclose(odt.odt_to_ri(f=f[0], res=res, nm=nm), ri[0])
    ri = odt.opt_to_ri(f=f, res=res, nm=nm)
    assert np.allclose(np.array(ri).flatten().view(float), z["test_opt_to_ri"])
    assert np.allclose(odt.opt_to_ri(f=f[0], res=res, nm=nm), ri[0])


def test_ri_complex_and_single_precision(cuda_ready):
    import torch
    import odtbrain_gb300 as odt
    rng = np.random.default_rng(2)
    f = (rng.normal(0, 3, (7, 9, 11)) + 1j * rng.normal(0, 3, (7, 9, 11)))
    f[0, 0, 0] = -50 + 0j   # negative real argument: root on the imaginary axis
    for res, nm in ((3.0, 1.333), (2.1, 1.34)):
        for fn in ("odt_to_ri", "opt_to_ri"):
            ref = getattr(O, fn)(f, res, nm)
            got = getattr(odt, fn)(f, res, nm)
            assert got.dtype == np.complex128
            assert np.abs(got - ref).max() <= 1e-14 * np.abs(ref).max()
            got32 = getattr(odt, fn)(f.astype(np.complex64), res, nm)
            assert got32.dtype == np.complex64
            assert np.abs(got32 - ref).max() <= 1e-6 * np.abs(ref).max()
            t = getattr(odt, fn)(torch.tensor(f, device=cuda_ready), res, nm)
            assert t.is_cuda and np.allclose(t.cpu().numpy(), ref)
    # real data below -km^2: NaN, like NumPy
    with np.errstate(invalid="ignore"):
        ref = O.odt_to_ri(np.array([-1e6, 0.5]), 3.0, 1.333)
    got = odt.odt_to_ri(np.array([-1e6, 0.5]), 3.0, 1.333)
    assert np.isnan(got[0]) and np.isclose(got[1], ref[1].real)


@pytest.mark.parametrize("n", [1, 2, 3, 4, 5, 7, 1023, 4097])
def test_ri_vector_and_tail_paths(cuda_ready, n):
    """Single-precision conversions take 16-byte accesses on aligned data
    with a scalar tail, and the scalar kernel on data that is not 16-byte
    aligned (a tensor view one element in): every path against the
    oracle."""
    import torch
    import odtbrain_gb300 as odt
    rng = np.random.default_rng(n)
    base = rng.normal(0, 3, n + 1) + 1j * rng.normal(0, 3, n + 1)
    for res, nm in ((3.0, 1.333),):
        for fn in ("odt_to_ri", "opt_to_ri"):
            for data in (base.astype(np.complex64),
                         np.abs(base.real).astype(np.float32)):
                ref = getattr(O, fn)(data[1:].astype(
                    np.complex128 if data.dtype.kind == "c" else np.float64),
                    res, nm)
                scale = np.abs(ref).max()
                t = torch.tensor(data, device=cuda_ready)
                for view in (t[1:], t[1:].clone()):
                    got = getattr(odt, fn)(view, res, nm).cpu().numpy()
                    assert got.dtype == data.dtype
                    assert np.abs(got - ref).max() <= 1e-6 * scale, \
                        (fn, data.dtype, view.data_ptr() % 16)
