"""Import shims that let the unmodified ODTbrain reference run in a container
that lacks pyFFTW, numexpr and scikit-image.

Used only by ``make_golden.py`` (fixture generation, run where the reference
source tree is mounted).  Nothing in the package, the GPU tests, ``smoke()``
or ``bench.py`` imports this module.

The stand-ins follow the behaviour the reference relies on:

* ``pyfftw.FFTW(a, b, axes, direction).execute()`` -- FFTW's ``execute`` is
  unnormalised in both directions (``_alg3d_bpp.py:460-478, 507, 527``); the
  backward stand-in therefore uses ``scipy.fft.ifftn(..., norm="forward")``.
* ``numexpr.evaluate(expr, local_dict, casting, out)`` -- evaluated with
  NumPy (``_alg3d_bpp.py:434-437, 518-523``).
* ``skimage.restoration.unwrap_phase`` -- raises, unless a restatement is
  installed in ``UNWRAP_PHASE`` (make_golden.py installs the oracle's, to
  run the reference's 3D ``sinogram_as_rytov`` around it).
* ``FFTW.N`` -- the number of transformed elements, which ``apple.correct``
  divides by (odtbrain/apple.py:243).
"""
import os
import sys
import types

import numpy as np
import scipy.fft

# Root of the reference source tree (the directory holding ``odtbrain/``),
# from the environment; load_reference() refuses to guess it.
REFERENCE_ROOT = os.environ.get("ODT_REFERENCE_ROOT")


def _make_pyfftw():
    mod = types.ModuleType("pyfftw")

    def empty_aligned(shape, dtype=np.float64, order="C", n=None):
        return np.empty(shape, dtype=dtype, order=order)

    class FFTW:
        def __init__(self, input_array, output_array, axes=(-1,),
                     direction="FFTW_FORWARD", flags=(), threads=1,
                     planning_timelimit=None):
            self.input_array = input_array
            self.output_array = output_array
            self.axes = tuple(axes)
            self.direction = direction
            self.N = int(np.prod([input_array.shape[a] for a in self.axes]))

        def execute(self):
            if self.direction == "FFTW_FORWARD":
                res = scipy.fft.fftn(self.input_array, axes=self.axes)
            else:
                res = scipy.fft.ifftn(self.input_array, axes=self.axes,
                                      norm="forward")
            self.output_array[...] = res

        def __call__(self):
            self.execute()
            return self.output_array

    mod.empty_aligned = empty_aligned
    mod.FFTW = FFTW
    return mod


def _make_numexpr():
    mod = types.ModuleType("numexpr")

    def set_num_threads(n):
        return 1

    def evaluate(expr, local_dict=None, casting="safe", out=None, **kw):
        env = {"exp": np.exp, "sqrt": np.sqrt, "abs": np.abs}
        env.update(local_dict or {})
        res = eval(expr, {"__builtins__": {}}, env)
        if out is not None:
            out[...] = res
            return out
        return res

    mod.set_num_threads = set_num_threads
    mod.evaluate = evaluate
    return mod


# Stand-in for skimage.restoration.unwrap_phase(image, rng=...): None
# raises; make_golden.py installs the oracle's restatement
# (oracle/unwrap_oracle.py:unwrap_2d) to run the reference's 3D
# sinogram_as_rytov / sinogram_as_radon around it.
UNWRAP_PHASE = [None]


def _make_skimage():
    sk = types.ModuleType("skimage")
    rest = types.ModuleType("skimage.restoration")

    def unwrap_phase(image, wrap_around=False, rng=None, **kwargs):
        if UNWRAP_PHASE[0] is None:
            raise NotImplementedError("scikit-image is not installed")
        return UNWRAP_PHASE[0](np.asarray(image, dtype=np.float64))

    rest.unwrap_phase = unwrap_phase
    sk.restoration = rest
    return sk, rest


def load_reference():
    """Return the reference ``odtbrain`` module, imported read-only from
    $ODT_REFERENCE_ROOT."""
    if not REFERENCE_ROOT or not os.path.isdir(
            os.path.join(REFERENCE_ROOT, "odtbrain")):
        raise RuntimeError(
            "set ODT_REFERENCE_ROOT to the ODTbrain source tree (the "
            "directory that contains odtbrain/); got %r" % (REFERENCE_ROOT,))
    sys.dont_write_bytecode = True
    if "odtbrain" in sys.modules and hasattr(sys.modules["odtbrain"],
                                             "backpropagate_3d"):
        return sys.modules["odtbrain"]
    sys.modules.setdefault("pyfftw", _make_pyfftw())
    sys.modules.setdefault("numexpr", _make_numexpr())
    sk, rest = _make_skimage()
    sys.modules.setdefault("skimage", sk)
    sys.modules.setdefault("skimage.restoration", rest)
    ver = types.ModuleType("odtbrain._version")
    ver.version = "0.4.12+shim"
    sys.modules["odtbrain._version"] = ver
    if REFERENCE_ROOT not in sys.path:
        sys.path.insert(0, REFERENCE_ROOT)
    import odtbrain  # noqa: E402
    return odtbrain
