"""CPU tests: the FP64 oracle of the 2D path and of the refractive-index
conversions against the reference's own golden vectors
(tests/data/alg2d_bpp__*.zip, processing__test_{odt,opt}_to_ri.zip, re-saved
in tests/golden/reference_zips.npz) and against outputs of the unmodified
reference (tests/golden/reference_cases.npz)."""
import numpy as np
import pytest

from oracle import odt_oracle as O
from sino_gen import cutout, gauss_sino_2d, parameter_sets


@pytest.mark.parametrize("name,ampl", [("test_2d_backprop_phase", (1., 1.)),
                                       ("test_2d_backprop_full", (.9, 1.1))])
def test_oracle_2d_reference_zips(golden, name, ampl):
    sino, angles = gauss_sino_2d(ampl_range=ampl)
    r = [cutout(O.backpropagate_2d(sino, angles, **p))
         for p in parameter_sets(2)]
    got = np.array(r).flatten().view(float)
    ref = golden["reference_zips"][name]
    assert np.allclose(got, ref, rtol=0, atol=1e-9 * np.abs(ref).max())


def test_oracle_2d_reference_cases(golden):
    from conftest import reference_cases
    cases = list(reference_cases(golden, two_d=True))
    assert len(cases) == 5
    for n, sino, angles, kw, ref in cases:
        out = O.backpropagate_2d(sino, angles, **kw)
        assert out.shape == ref.shape and out.dtype == ref.dtype, n
        err = np.abs(out - ref).max() / np.abs(ref).max()
        assert err < 1e-11, (n, err)


def _ri_data():
    ln = 10
    f = np.arange(ln ** 3).reshape(ln, ln, ln)
    return f + np.linspace(1, 2, ln), 7, 1.34


def test_oracle_ri_reference_zips(golden):
    f, res, nm = _ri_data()
    z = golden["reference_zips"]
    ri = O.odt_to_ri(f, res, nm)
    assert np.allclose(np.array(ri.real).flatten(), z["test_odt_to_ri"])
    ri = O.opt_to_ri(f, res, nm)
    assert np.allclose(np.array(ri).flatten(), z["test_opt_to_ri"])
