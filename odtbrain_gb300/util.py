"""Angular weighting (FP64, host side).

Mirrors ``odtbrain.util.compute_angle_weights_1d`` (odtbrain/util.py:4-67).
"""
import numpy as np


def compute_angle_weights_1d(angles):
    """Weights proportional to the angular gap around each projection.

    Angles are wrapped modulo pi relative to the smallest angle; each
    distinct angle gets ``(next - previous) mod pi`` (over the sorted distinct
    angles, cyclically), shared equally by its duplicates, and the weights
    are normalised to mean one.  Same arithmetic, in the same order, as
    odtbrain/util.py:51-67, so the FP64 result is identical.
    """
    angles = np.asarray(angles)
    flat = (angles.flatten() - np.min(angles)) % np.pi
    distinct, back, counts = np.unique(flat, return_inverse=True,
                                       return_counts=True)
    order = np.argsort(distinct)
    ordered = distinct[order]
    gap = (np.roll(ordered, -1) - np.roll(ordered, 1)) % np.pi
    gap_sum = np.sum(gap)
    gap /= counts[order]
    w_sorted = gap / gap_sum * flat.size
    w_distinct = np.zeros_like(w_sorted)
    w_distinct[order] = w_sorted
    return w_distinct[back]
