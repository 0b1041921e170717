"""Cases of reference_apple_helpers.npz (written by make_golden.py from the
reference's constraint_nn, constraint_sh and envelope_gauss,
odtbrain/apple.py:56-110 and :289-350), for the CPU and GPU tests."""
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))


def load():
    with np.load(os.path.join(HERE, "reference_apple_helpers.npz")) as z:
        return {k: z[k] for k in z.files}


def constraint_cases(fx):
    """(name, function name, input, keyword arguments, reference output);
    the input is in_<src> cast to the output's dtype (its real part for a
    real type), as make_golden.py made it."""
    for n in sorted({k.split("__")[0] for k in fx if k.endswith("__fn")}):
        ref = fx[n + "__out"]
        src = fx["in_" + str(fx[n + "__src"])]
        if np.iscomplexobj(ref):
            data = src.astype(ref.dtype)
        else:
            data = np.ascontiguousarray(src.real.astype(ref.dtype))
        kw = {}
        if n + "__mask" in fx:
            kw["mask"] = fx[n + "__mask"]
        if n + "__shell" in fx:
            kw["bg_shell"] = fx[n + "__shell"]
        yield n, str(fx[n + "__fn"]), data, kw, ref


def envelope_cases(fx):
    """(name, spectrum, core, reference envelope)."""
    for n in sorted({k.split("__")[0] for k in fx if k.startswith("env_")}):
        yield n, fx[n + "__ft"], fx[n + "__core"], fx[n + "__out"]
