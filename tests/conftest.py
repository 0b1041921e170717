import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
for p in (ROOT, GOLDEN):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line(
        "markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built "
        "odtbrain_gb300 library")


@pytest.fixture(scope="session")
def golden():
    """Fixtures written by tests/golden/make_golden.py from the reference."""
    out = {}
    for name in ("reference_zips", "reference_cases", "reference_geometry"):
        with np.load(os.path.join(GOLDEN, name + ".npz")) as z:
            out[name] = {k: z[k] for k in z.files}
    return out


@pytest.fixture(scope="session")
def cuda_ready():
    import torch
    if not torch.cuda.is_available():
        pytest.fail("GPU test selected but no CUDA device is visible")
    import odtbrain_gb300.build as b
    b.build()
    return torch.device("cuda", 0)


def reference_cases(golden, two_d=False):
    """(name, sino, angles, kwargs, out) of the reference-made 3D cases, or
    of the 2D cases (names b2d_*) with ``two_d``."""
    cases = golden["reference_cases"]
    names = sorted({k.split("__")[0] for k in cases
                    if k.startswith("b2d_") == two_d})
    for n in names:
        kw = json.loads(str(cases[n + "__kw"]))
        if "padding" in kw and not two_d:
            kw["padding"] = tuple(kw["padding"])
        yield n, cases[n + "__sino"], cases[n + "__angles"], kw, \
            cases[n + "__out"]


def reference_c1():
    """The whole 60-angle 64^3 workload and the reference's output for it
    (tests/golden/reference_c1.npz, written by make_golden.py): returns
    (sino, angles, kwargs, out) with the input regenerated by the seeded
    phantom generator and checked against the stored checksum."""
    from sino_gen import ellipsoid_phantom_sinogram
    with np.load(os.path.join(GOLDEN, "reference_c1.npz")) as z:
        args = json.loads(str(z["args"]))
        kw = json.loads(str(z["kw"]))
        out = z["out_re"].astype(np.float64) + 1j * z["out_im"]
        abs_sum = float(z["input_abs_sum"])
        angles_ref = z["angles"]
    args["count_range"] = tuple(args["count_range"])
    args["semi_range"] = tuple(args["semi_range"])
    sino, angles = ellipsoid_phantom_sinogram(**args)
    assert abs(np.abs(sino).sum() - abs_sum) <= 1e-12 * abs_sum
    np.testing.assert_array_equal(angles, angles_ref)
    return sino, angles, kw, out
