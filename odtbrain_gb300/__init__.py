"""GB300-native (sm_103a) 3D filtered backpropagation for optical
diffraction tomography.

Drop-in replacements for ``odtbrain.backpropagate_3d`` and
``odtbrain.backpropagate_3d_tilted``: the same signatures and semantics,
with the per-angle filter, propagation, spline resampling and accumulation
running in hand-written CUDA kernels behind a C ABI
(``include/odtbrain_gb300.h``).
"""
from ._alg3d import backpropagate_3d, backpropagate_3d_tilted  # noqa: F401
from . import util  # noqa: F401

__version__ = "0.1.0"
