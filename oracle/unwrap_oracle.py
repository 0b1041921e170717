"""TEST INFRASTRUCTURE ONLY -- CPU oracle for ODTbrain's sinogram
preparation: ``sinogram_as_rytov`` / ``sinogram_as_radon`` and their helpers
(odtbrain/_prepare_sino.py:7-182).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` may import this module; the product never calls it.

What the reference computes, per step:

* ``phi = angle(uSin / u0)``, ``lna = log(|uSin / u0|)`` in the precision of
  ``result_type(uSin, u0)`` (_prepare_sino.py:159-162);
* 2D sinograms (A, N): ``numpy.unwrap`` along the detector axis
  (_prepare_sino.py:164-166) -- NumPy is present, so this oracle calls it;
* 3D sinograms (A, Ny, Nx): ``skimage.restoration.unwrap_phase(phi[a],
  rng=47)`` per angle (_prepare_sino.py:167-172).  scikit-image
  (pinned ``scikit-image>=0.21.0,<1``) is not installed; :func:`unwrap_2d`
  below restates the algorithm it implements, Herraez et al., "Fast
  two-dimensional phase-unwrapping algorithm based on sorting by
  reliability following a noncontinuous path", Appl. Opt. 41, 7437 (2002),
  in the form of scikit-image's implementation: pixel reliability = sum of
  the squared wrapped second differences (horizontal, vertical, both
  diagonals) for interior pixels, a large pseudo-random value for border
  pixels; edge weight = sum of its two pixels' values; edges unwrapped in
  ascending weight order, each joining two groups, the smaller group (by
  pixel count) shifted by whole turns to match the larger;
* ``align_unwrapped`` (_prepare_sino.py:7-46) and ``divmod_neg``
  (_prepare_sino.py:49-57), restated with NumPy / SciPy as the reference
  calls them;
* output ``u0 * (1j * phi + lna)`` (rytov) or ``phi`` (radon).

Where this restatement cannot follow the reference exactly:

* border reliabilities: scikit-image draws them from the C library's
  ``rand()`` seeded from its ``rng`` argument; here they come from
  :func:`border_noise` (a fixed integer hash of (seed, pixel index)), the
  same function the GPU kernels use;
* ties between equal edge weights: scikit-image's quicksort order is not
  specified; here ties go by the edge's creation index (all horizontal edges
  row-major, then all vertical edges row-major).

With distinct weights the unwrapping tree is the unique minimum spanning
tree of the edge weights, so interior results do not depend on either
point; for residue-free phase maps (every 2x2 loop of wrapped differences
sums to zero) no result depends on them.  The reference's golden vectors
(tests/data/processing__test_sino_{rytov,radon}.zip) pin this oracle.
"""
import numpy as np
import scipy.stats

TWOPI = 2 * np.pi
BORDER_BASE = 9999999.0
DEFAULT_SEED = 47


def border_noise(seed, n):
    """Pseudo-random integers in [0, 2**31) for pixel indices ``n`` (array):
    a splitmix64 finaliser of ``seed * 0x9E3779B97F4A7C15 + (n + 1) *
    0xBF58476D1CE4E5B9`` (mod 2**64), top 31 bits."""
    m = (1 << 64) - 1
    n = np.asarray(n, dtype=np.uint64)
    with np.errstate(over="ignore"):
        x = (np.uint64((seed * 0x9E3779B97F4A7C15) & m)
             + (n + np.uint64(1)) * np.uint64(0xBF58476D1CE4E5B9))
        x ^= x >> np.uint64(30)
        x *= np.uint64(0xBF58476D1CE4E5B9)
        x ^= x >> np.uint64(27)
        x *= np.uint64(0x94D049BB133111EB)
        x ^= x >> np.uint64(31)
    return (x >> np.uint64(33)).astype(np.int64)


def _wrap(d):
    """Wrap a phase difference into [-pi, pi] (values beyond one turn are
    moved by one turn)."""
    d = np.array(d, dtype=np.float64, copy=True)
    d[d > np.pi] -= TWOPI
    d[d < -np.pi] += TWOPI
    return d


def pixel_reliability(phi, seed=DEFAULT_SEED):
    """Reliability value of every pixel of a 2D wrapped phase map (smaller is
    more reliable): H^2 + V^2 + D1^2 + D2^2 of the wrapped second
    differences inside, ``9999999 + border_noise`` on the border."""
    p = np.asarray(phi, dtype=np.float64)
    H, W = p.shape
    rel = BORDER_BASE + border_noise(seed, np.arange(H * W)).reshape(H, W) \
        .astype(np.float64)
    if H >= 3 and W >= 3:
        c = p[1:-1, 1:-1]
        h = _wrap(p[1:-1, :-2] - c) - _wrap(c - p[1:-1, 2:])
        v = _wrap(p[:-2, 1:-1] - c) - _wrap(c - p[2:, 1:-1])
        d1 = _wrap(p[:-2, :-2] - c) - _wrap(c - p[2:, 2:])
        d2 = _wrap(p[:-2, 2:] - c) - _wrap(c - p[2:, :-2])
        rel[1:-1, 1:-1] = ((h * h + v * v) + d1 * d1) + d2 * d2
    return rel


def edge_list(H, W, rel):
    """(pixel1, pixel2, weight) of the grid edges in creation order:
    horizontal edges row-major, then vertical edges row-major."""
    idx = np.arange(H * W).reshape(H, W)
    p1 = np.concatenate([idx[:, :-1].ravel(), idx[:-1, :].ravel()])
    p2 = np.concatenate([idx[:, 1:].ravel(), idx[1:, :].ravel()])
    r = rel.ravel()
    return p1, p2, r[p1] + r[p2]


def _find_wrap(v1, v2):
    d = v1 - v2
    if d > np.pi:
        return -1
    if d < -np.pi:
        return 1
    return 0


def unwrap_2d(phi, seed=DEFAULT_SEED, return_head=False, anchor="head"):
    """Reliability-sorted unwrapping of one 2D phase map (FP64 result).

    Edges are processed in ascending (weight, creation index) order.  For
    edge (p1, p2) with ``e = find_wrap(phi[p1], phi[p2])`` the unwrapped
    values satisfy ``k[p2] = k[p1] - e``.  Merging follows the reference
    implementation's rules: a lone p2 joins p1's group; else a lone p1 joins
    p2's group; else the group of p2 joins p1's group when p1's group is
    strictly larger, otherwise p1's group joins p2's.  The pixel that heads
    the final group keeps its wrapped value (``anchor="head"``, the
    reference's choice), or pixel 1 of the first edge does
    (``anchor="first_edge"``, the GPU product's choice)."""
    p = np.asarray(phi, dtype=np.float64)
    H, W = p.shape
    n = H * W
    vals = p.ravel()
    rel = pixel_reliability(p, seed)
    e1, e2, w = edge_list(H, W, rel)
    order = np.lexsort((np.arange(w.size), w))
    head = np.arange(n)
    members = [[i] for i in range(n)]
    inc = np.zeros(n, dtype=np.int64)
    for k in order:
        a, b = int(e1[k]), int(e2[k])
        ha, hb = head[a], head[b]
        if ha == hb:
            continue
        e = _find_wrap(vals[a], vals[b])
        if len(members[hb]) == 1:
            keep, gone, delta = ha, hb, inc[a] - e - inc[b]
        elif len(members[ha]) == 1:
            keep, gone, delta = hb, ha, inc[b] + e - inc[a]
        elif len(members[ha]) > len(members[hb]):
            keep, gone, delta = ha, hb, inc[a] - e - inc[b]
        else:
            keep, gone, delta = hb, ha, inc[b] + e - inc[a]
        for m in members[gone]:
            head[m] = keep
            inc[m] += delta
        members[keep].extend(members[gone])
        members[gone] = []
    if anchor == "first_edge" and order.size:
        inc = inc - inc[int(e1[order[0]])]
    out = (vals + TWOPI * inc.astype(np.float64)).reshape(H, W)
    if return_head:
        return out, int(head[0])
    return out


def first_edge_pixel(phi, seed=DEFAULT_SEED):
    """Pixel 1 of the first edge in (weight, creation index) order: the
    pixel that heads the first group formed."""
    p = np.asarray(phi, dtype=np.float64)
    H, W = p.shape
    e1, _e2, w = edge_list(H, W, pixel_reliability(p, seed))
    k = np.lexsort((np.arange(w.size), w))[0]
    return int(e1[k])


def divmod_neg(a, b):
    """divmod with the remainder closest to zero (_prepare_sino.py:49-57)."""
    q, r = divmod(a, b)
    sr = np.sign(r)
    if np.abs(r) > b / 2:
        q += sr
        r -= b * sr
    return q, r


def align_unwrapped(sino):
    """In place: remove per-angle whole-turn steps (majority vote of five
    border samples unwrapped along the angle axis), then the whole turns of
    the global minimum (_prepare_sino.py:7-46)."""
    samples = []
    if sino.ndim == 2:
        for c in (0, 1, 2, -1, -2):
            samples.append(sino[:, c])
    else:
        for (y, x) in ((0, 0), (0, -1), (-1, 0), (-1, -1), (0, 1)):
            samples.append(sino[:, y, x])
    steps = np.zeros((len(samples), samples[0].shape[0]))
    for i, s in enumerate(samples):
        steps[i] = s - np.unwrap(s)
    remove = scipy.stats.mode(steps, axis=0, keepdims=True)[0][0]
    minimum = divmod_neg(np.min(sino), TWOPI)[0]
    remove += minimum * TWOPI
    for i in range(len(sino)):
        sino[i] -= remove[i]


def _unwrap_phase_map(phi, seed, anchor):
    if phi.ndim == 2:
        phi[:] = np.unwrap(phi, axis=-1)
    else:
        for a in range(len(phi)):
            phi[a] = unwrap_2d(phi[a], seed, anchor=anchor)
    return phi


def sinogram_as_rytov(uSin, u0=1, align=True, seed=DEFAULT_SEED,
                      anchor="head"):
    """Rytov sinogram ``u0 * (lna + 1j*phi)`` (_prepare_sino.py:105-182)."""
    q = uSin / u0
    phi = np.angle(q)
    lna = np.log(np.absolute(q))
    _unwrap_phase_map(phi, seed, anchor)
    if align:
        align_unwrapped(phi)
    return u0 * (1j * phi + lna)


def sinogram_as_radon(uSin, align=True, seed=DEFAULT_SEED, anchor="head"):
    """Unwrapped phase sinogram (_prepare_sino.py:60-102)."""
    phi = np.angle(uSin)
    _unwrap_phase_map(phi, seed, anchor)
    if align:
        align_unwrapped(phi)
    return phi
