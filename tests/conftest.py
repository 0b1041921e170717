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
