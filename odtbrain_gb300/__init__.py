"""GB300-native (sm_103a) filtered backpropagation for optical diffraction
tomography.

Drop-in replacements for ``odtbrain.backpropagate_3d``,
``odtbrain.backpropagate_3d_tilted`` and ``odtbrain.backpropagate_2d`` (the
same signatures and semantics, with the per-angle filter, propagation,
spline resampling and accumulation running in hand-written CUDA kernels
behind a C ABI, ``include/odtbrain_gb300.h``), and for the refractive-index
conversions ``odt_to_ri`` / ``opt_to_ri``, and for the sinogram preparation
``sinogram_as_rytov`` / ``sinogram_as_radon`` (GPU phase unwrapping), and
the missing-apple-core correction ``apple.correct``.
"""
from ._alg2d import backpropagate_2d  # noqa: F401
from ._alg3d import backpropagate_3d, backpropagate_3d_tilted  # noqa: F401
from ._prepare_sino import sinogram_as_radon, sinogram_as_rytov  # noqa: F401
from ._translate_ri import odt_to_ri, opt_to_ri  # noqa: F401
from . import apple  # noqa: F401
from . import util  # noqa: F401
from . import warn  # noqa: F401

__version__ = "0.1.0"
