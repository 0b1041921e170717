"""Test inputs for the parity tests.

* ``gauss_sino_2d`` / ``gauss_sino_3d`` / ``gauss_sino_3d_tilted`` /
  ``parameter_sets`` / ``cutout`` restate the reference's test helpers
  (tests/common_methods.py:10-60, 63-118, 121-184, 231-243, 187-205) so the GPU
  tests can rebuild the exact inputs of the reference's own tests and of the
  fixtures without the reference tree.  ``cutout`` keeps the reference's
  quirk (its z mask reuses the y axis, common_methods.py:200) because the
  reference's golden vectors were written with it.
* ``ellipsoid_phantom_sinogram`` builds the seeded synthetic workloads of the
  benchmark configurations: random ellipsoids inside the inscribed sphere,
  analytic line integrals of (n - nm) along the beam for each rotation about
  the (possibly tilted) axis, Rytov-form data ``a + i*phi``.
"""
import numpy as np


def _normalize(av, vmin=0., vmax=1.):
    if vmin == vmax:
        return np.ones_like(av) * vmin
    if vmax < vmin:
        vmin, vmax = vmax, vmin
    unit = (av - np.min(av)) / (np.max(av) - np.min(av))
    return unit * (vmax - vmin) + vmin


def _gauss_frames(A, Nx, Ny, max_phase, ampl_range):
    angles = np.linspace(0, 2 * np.pi, A, endpoint=False)
    x = np.linspace(-Nx / 2, Nx / 2, Nx, endpoint=True).reshape(1, -1)
    y = np.linspace(-Ny / 2, Ny / 2, Ny, endpoint=True).reshape(-1, 1)
    dev = min(np.sqrt(Nx / 2), np.sqrt(Ny / 2))
    off = Nx / 7
    for ii in range(A):
        x0 = np.cos(angles[ii]) * off
        phase = np.exp(-(x - x0) ** 2 / dev ** 2) * np.exp(-y ** 2 / dev ** 2)
        phase = _normalize(phase, vmax=max_phase)
        if ampl_range[0] == ampl_range[1]:
            ampl = None
        else:
            adev = dev / 5
            aoff = off * .3
            ring = (np.exp(-(x - x0 - aoff) ** 2 / adev ** 2)
                    + np.exp(-(x - x0 + aoff) ** 2 / adev ** 2))
            ampl = _normalize(ring, vmin=ampl_range[0], vmax=ampl_range[1])
        yield ii, angles, phase, ampl


def gauss_sino_2d(A=9, N=22, max_phase=5.0, ampl_range=(1.0, 1.0)):
    """2D variant: an off-centre Gaussian phase line per angle, amplitude 1
    or a normalised double ring (tests/common_methods.py:10-60)."""
    out = np.zeros((A, N), dtype=np.complex128)
    angles = np.linspace(0, 2 * np.pi, A, endpoint=False)
    x = np.linspace(-N / 2, N / 2, N, endpoint=True)
    dev = np.sqrt(N / 2)
    off = N / 7
    for ii in range(A):
        x0 = np.cos(angles[ii]) * off
        phase = _normalize(np.exp(-(x - x0) ** 2 / dev ** 2), vmax=max_phase)
        if ampl_range[0] == ampl_range[1]:
            ampl = ampl_range[0]
        else:
            adev = dev / 5
            aoff = off * .3
            ring = (np.exp(-(x - x0 - aoff) ** 2 / adev ** 2)
                    + np.exp(-(x - x0 + aoff) ** 2 / adev ** 2))
            ampl = _normalize(ring, vmin=ampl_range[0], vmax=ampl_range[1])
        out[ii] = ampl * np.exp(1j * phase)
    return out, angles


def gauss_sino_3d(A=9, Nx=22, Ny=22, max_phase=5.0, ampl_range=(1.0, 1.0)):
    """Off-centre Gaussian phase rotating about y; returns (sino, angles)."""
    out = np.zeros((A, Ny, Nx), dtype=np.complex128)
    angles = None
    for ii, angles, phase, ampl in _gauss_frames(A, Nx, Ny, max_phase,
                                                 ampl_range):
        a = ampl_range[0] if ampl is None else ampl
        out[ii] = a * np.exp(1j * phase)
    return out, angles


def gauss_sino_3d_tilted(A=9, Nx=22, Ny=22, max_phase=5.0,
                        ampl_range=(1.0, 1.0), tilt_plane=0.0):
    """As gauss_sino_3d, each frame rotated in-plane by ``tilt_plane``."""
    from scipy.ndimage import rotate
    out = np.zeros((A, Ny, Nx), dtype=np.complex128)
    angles = None
    for ii, angles, phase, ampl in _gauss_frames(A, Nx, Ny, max_phase,
                                                 ampl_range):
        if ampl is None:
            ampl = np.ones((Nx, Ny)) * ampl_range[0]
        ampl = rotate(ampl, np.rad2deg(tilt_plane), reshape=False, cval=1)
        phase = rotate(phase, np.rad2deg(tilt_plane), reshape=False, cval=0)
        out[ii] = ampl * np.exp(1j * phase)
    return out, angles


def parameter_sets(n=1):
    res, lD, nm = 2.1, 0, 1.333
    out = []
    for _ in range(n):
        out.append({"res": res, "lD": lD, "nm": nm})
        res += .1
        lD += np.pi
        nm *= 1.01
    return out


def cutout(a):
    """Zero everything outside the reference test's mask (see module doc);
    2D arrays get the disc mask."""
    a = np.array(a, copy=True)
    n = a.shape[0]
    c = n / 2
    if a.ndim == 2:
        x = np.arange(n).reshape(-1, 1)
        y = x.reshape(1, -1)
        a *= ((x - c) ** 2 + (y - c) ** 2) < c ** 2
        return a
    x = np.arange(n).reshape(-1, 1, 1)
    y = x.reshape(1, -1, 1)
    mask = ((x - c) ** 2 + (y - c) ** 2 + (y - c) ** 2) < c ** 2
    a *= mask
    return a


# ------------------------------------------------------------ phantoms
def random_ellipsoids(rng, n, count_range, semi_range, nm=1.333,
                      dn_range=(1.335, 1.36)):
    """Seeded ellipsoids inside the inscribed sphere of an n^3 volume.
    Each: centre c (voxels, relative to the volume centre), semi-axes s,
    rotation R (columns are the ellipsoid axes), refractive index."""
    count = int(rng.integers(count_range[0], count_range[1] + 1))
    ells = []
    for _ in range(count):
        s = rng.uniform(semi_range[0], semi_range[1], 3)
        rmax = max(0.0, n / 2 - 1 - s.max())
        while True:
            c = rng.uniform(-rmax, rmax, 3)
            if np.linalg.norm(c) <= rmax:
                break
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w),
                       2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z),
                       2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w),
                       1 - 2 * (x * x + y * y)]])
        ells.append((c, s, R, rng.uniform(dn_range[0], dn_range[1])))
    return ells


def _rotation_about(axis, t):
    axis = np.asarray(axis, float)
    axis = axis / np.linalg.norm(axis)
    K = np.array([[0, -axis[2], axis[1]], [axis[2], 0, -axis[0]],
                  [-axis[1], axis[0], 0]])
    return np.eye(3) + np.sin(t) * K + (1 - np.cos(t)) * (K @ K)


def ellipsoid_phantom_sinogram(n, A, seed, count_range, semi_range,
                               res=3.0, nm=1.333, axis=(0, 1, 0),
                               amp_sigma=0.1, angles=None, ny=None):
    """Rytov sinogram (A, ny, n) complex128 and angles for a seeded
    ellipsoid phantom.

    Detector pixel (y, x) looks along +z through the phantom rotated by
    angle phi about ``axis`` (x, y, z order).  The phase is
    (2 pi / res) * integral (n - nm) dz (res = wavelength in pixels), the
    log-amplitude is N(0, amp_sigma); the returned data is a + i*phase.
    """
    rng = np.random.default_rng(seed)
    ny = n if ny is None else ny
    ells = random_ellipsoids(rng, n, count_range, semi_range, nm)
    if angles is None:
        angles = np.linspace(0, 2 * np.pi, A, endpoint=False)
    xs = np.arange(n) - (n - 1) / 2
    ys = np.arange(ny) - (ny - 1) / 2
    X, Y = np.meshgrid(xs, ys, indexing="xy")
    k0 = 2 * np.pi / res
    sino = np.zeros((len(angles), ny, n), dtype=np.complex128)
    for ia, phi in enumerate(angles):
        Rphi = _rotation_about(axis, phi)
        path = np.zeros((ny, n))
        for c, s, R, nidx in ells:
            # ellipsoid in the rotated frame: centre Rphi c, axes Rphi R
            cr = Rphi @ c
            Rr = Rphi @ R
            # ray p(t) = (X, Y, t): solve |S^-1 Rr^T (p - cr)|^2 = 1
            Q = Rr @ np.diag(1.0 / s ** 2) @ Rr.T
            d = np.stack([X - cr[0], Y - cr[1]], axis=-1)
            qa = Q[2, 2]
            qb = 2 * (d[..., 0] * Q[0, 2] + d[..., 1] * Q[1, 2])
            qc = (Q[0, 0] * d[..., 0] ** 2 + 2 * Q[0, 1] * d[..., 0]
                  * d[..., 1] + Q[1, 1] * d[..., 1] ** 2 - 1)
            disc = qb * qb - 4 * qa * qc
            chord = np.where(disc > 0, np.sqrt(np.maximum(disc, 0)) / qa, 0)
            path += chord * (nidx - nm)
        phase = k0 * path
        logamp = rng.normal(0, amp_sigma, (ny, n))
        sino[ia] = logamp + 1j * phase
    return sino, np.asarray(angles)
