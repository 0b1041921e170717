"""FP64 host setup of the 3D backpropagation.

Everything here runs once per call on the host in double precision and is
written so that its floating-point operations happen in the same order as the
reference's, which makes the constants handed to the GPU bit-identical to the
reference's FP64 values:

* padding sizes        odtbrain/_alg3d_bpp.py:285-304
* filter and phase     odtbrain/_alg3d_bpp.py:317, 371-399, 419-437
                       odtbrain/_alg3d_bppt.py:680, 737-771
* y-axis rotation      odtbrain/_alg3d_bpp.py:534, 73-81 and the matrix and
                       offset scipy.ndimage.rotate builds from them
* tilted geometry      odtbrain/_alg3d_bppt.py:26-371, 644-673, 863, 907-919
"""
import numpy as np
from scipy import special

from .util import compute_angle_weights_1d


def padded_size(n, padfac):
    """Second-next power of two of ``n*padfac``, at least 64."""
    return int(max(64., 2 ** np.ceil(np.log(n * padfac) / np.log(2))))


def padding_geometry(lny, lnx, padding, padfac):
    padx = padded_size(lnx, padfac) - lnx if padding[0] else 0
    pady = padded_size(lny, padfac) - lny if padding[1] else 0
    padyl = int(np.ceil(pady / 2))
    padxl = int(np.ceil(padx / 2))
    return dict(lNx=lnx + padx, lNy=lny + pady, padxl=padxl, padyl=padyl,
                padxr=padx - padxl, padyr=pady - padyl)


def _frequencies(lNx, lNy):
    kx = (2 * np.pi * np.fft.fftfreq(lNx)).reshape(1, -1)
    ky = (2 * np.pi * np.fft.fftfreq(lNy)).reshape(-1, 1)
    return kx, ky


def filter_tables(A, lNx, lNy, res, nm, lD, tilted_axis=None):
    """Return (filter, kz_phase) as contiguous FP64 arrays of shape
    (lNy, lNx): the complex factor the forward spectrum is multiplied by,
    ``prefactor [* filterabs] / (lNx*lNy)``, and ``km*(M-1)``, the
    propagator phase per unit z."""
    km = (2 * np.pi * nm) / res
    kx, ky = _frequencies(lNx, lNy)
    dphi0 = 2 * np.pi / A
    inside = (kx ** 2 + ky ** 2 < km ** 2)
    M = 1. / km * np.sqrt((km ** 2 - kx ** 2 - ky ** 2) * inside)
    pre = -1j * km / (2 * np.pi)
    pre *= dphi0
    if tilted_axis is None:
        pre *= np.abs(kx) * inside
        pre *= np.exp(-1j * km * (M - 1) * lD)
        filt = pre / (lNx * lNy)
    else:
        u, v, _w = tilted_axis
        gain = np.abs(kx * v + ky * u) * inside
        pre *= np.exp(-1j * km * (M - 1) * lD)
        filt = gain * pre / (lNx * lNy)
    filt = np.ascontiguousarray(np.broadcast_to(filt, (lNy, lNx)),
                                dtype=np.complex128)
    phase = np.ascontiguousarray(np.broadcast_to(km * (M - 1), (lNy, lNx)),
                                 dtype=np.float64)
    return filt, phase


# ------------------------------------------------------------- y-axis path
def rotation_y_geometry(angles, nz, nx):
    """Per angle: [m00, m01, m10, m11, off0, off1] of the plane rotation that
    ``scipy.ndimage.rotate(plane, -deg(phi), axes=(0, 2), reshape=False)``
    applies to a (nz, nx) plane (odtbrain/_alg3d_bpp.py:75, 534)."""
    angles = np.asarray(angles).reshape(-1)
    out = np.empty((angles.size, 6), dtype=np.float64)
    shape = np.asarray((nz, nx))
    center = (shape - 1) / 2
    for i, phi in enumerate(angles):
        deg = -np.rad2deg(phi)
        c, s = special.cosdg(deg), special.sindg(deg)
        mat = np.array([[c, s], [-s, c]])
        off = center - mat @ center
        out[i, :4] = mat.reshape(-1)
        out[i, 4:] = off
    return out


# ------------------------------------------------------------- tilted path
def norm_vec(vector):
    """Unit vector along ``vector`` (length-3)."""
    assert len(vector) == 3
    v = np.array(vector)
    return v / np.sqrt(np.sum(v ** 2))


def _rot_x(t):
    return np.array([[1, 0, 0],
                     [0, np.cos(t), -np.sin(t)],
                     [0, np.sin(t), np.cos(t)]])


def _rot_y_neg(t):
    # rotation by -t about y (x toward -z)
    return np.array([[np.cos(t), 0, -np.sin(t)],
                     [0, 1, 0],
                     [np.sin(t), 0, np.cos(t)]])


def _rot_z(t):
    return np.array([[np.cos(t), -np.sin(t), 0],
                     [np.sin(t), np.cos(t), 0],
                     [0, 0, 1]])


def sphere_points_from_angles_and_tilt(angles, tilted_axis):
    """Unit-sphere points of the projection directions for rotation angles
    about ``tilted_axis`` (reference axis [0, 1, 0]); the first angle maps
    to [0, 0, 1]."""
    assert len(angles.shape) == 1
    tilted_axis = norm_vec(tilted_axis)
    u, v, w = tilted_axis
    pts = np.zeros((angles.shape[0], 3), dtype=float)
    pts[:, 0] = np.sin(angles - angles[0])
    pts[:, 2] = np.cos(angles - angles[0])
    theta = np.arccos(v)
    if np.allclose(u, 0) and np.allclose(w, 0):
        phi = 0
    else:
        phi = np.arctan2(u, w)
    pts *= np.cos(theta)
    rx = _rot_x(theta)
    for i in range(pts.shape[0]):
        pts[i] = np.dot(rx, pts[i])
    pts = pts - (pts[0] - np.array([0, 0, 1])).reshape(1, 3)
    ry = np.array([[+np.cos(phi), 0, np.sin(phi)],
                   [0, 1, 0],
                   [-np.sin(phi), 0, np.cos(phi)]])
    for i in range(pts.shape[0]):
        pts[i] = np.dot(ry, pts[i])
    return pts


def rotate_points_to_axis(points, axis):
    """Rotate ``points`` about the origin so that ``axis`` becomes [0,1,0]
    (tilt toward y within the plane of ``axis`` and y)."""
    axis = norm_vec(axis)
    u, v, w = axis
    points = np.array(points)
    phi = np.arctan2(u, w)
    theta = np.arccos(v)
    rphi = _rot_y_neg(phi)
    rtheta = np.array([[1, 0, 0],
                       [0, np.cos(theta), np.sin(theta)],
                       [0, -np.sin(theta), np.cos(theta)]])
    dr = np.dot(rphi.T, np.dot(rtheta, rphi))
    out = np.zeros((len(points), 3))
    for i, pnt in enumerate(points):
        out[i] = np.dot(dr, pnt)
    return out


def rotation_matrix_from_point(point, ret_inv=False):
    """Rotation taking [0, 0, 1] to ``point`` (polar tilt, then azimuth
    about y), and optionally its inverse."""
    x, y, z = point
    phi = np.arctan2(x, z)
    theta = -np.arctan2(y, np.sqrt(x ** 2 + z ** 2))
    rtheta = _rot_x(theta)
    rphi = _rot_y_neg(phi)
    D = np.dot(rphi, rtheta)
    Dinv = np.dot(rtheta.T, rphi.T)
    if ret_inv:
        return D, Dinv
    return D


def rotation_matrix_from_point_planerot(point, plane_angle, ret_inv=False):
    """:func:`rotation_matrix_from_point` followed by an in-plane rotation
    by ``plane_angle`` about z."""
    D, Dinv = rotation_matrix_from_point(point, ret_inv=True)
    rz = _rot_z(plane_angle)
    DR = np.dot(D, rz)
    DRinv = np.dot(rz.T, Dinv)
    if ret_inv:
        return DR, DRinv
    return DR


def tilted_geometry(angles, tilted_axis, weight_angles, shape_xyz):
    """Weights (or None), per-angle [3x3 matrix row-major, offset] (A, 12)
    for the affine resampling of the (x, -y, z) slab, and the normalised
    axis.  Raises UserWarning-compatible behaviour is left to the caller."""
    angles = np.squeeze(np.array(angles, copy=True))
    tilted_axis = norm_vec(tilted_axis)
    angz = np.arctan2(tilted_axis[0], tilted_axis[1])
    rotmat = _rot_z(angz)
    axis_yz = norm_vec(np.dot(rotmat, tilted_axis))
    weights = None
    if len(angles.shape) == 1:
        if weight_angles:
            weights = compute_angle_weights_1d(angles)
        points = sphere_points_from_angles_and_tilt(angles, axis_yz)
    else:
        points = angles
        for i in range(points.shape[0]):
            points[i] = norm_vec(np.dot(rotmat, points[i]))
    points = rotate_points_to_axis(points=points, axis=axis_yz)
    c = 0.5 * np.array(shape_xyz) - .5
    geo = np.empty((points.shape[0], 12), dtype=np.float64)
    for i in range(points.shape[0]):
        _d, dinv = rotation_matrix_from_point_planerot(points[i],
                                                       plane_angle=angz,
                                                       ret_inv=True)
        geo[i, :9] = dinv.reshape(-1)
        geo[i, 9:] = c - np.dot(dinv, c)
    return weights, geo, tilted_axis


# ------------------------------------------------------------------ 2D path
def padding_geometry_2d(ln, padding):
    """Padded line length and left pad of the 2D algorithm
    (odtbrain/_alg2d_bpp.py:175-187): the next power of two of 2.1*ln, at
    least 64; left pad ceil(pad/2)."""
    order = max(64., 2 ** np.ceil(np.log(ln * 2.1) / np.log(2)))
    pad = order - ln if padding else 0
    padl = int(np.ceil(pad / 2))
    return dict(lN=int(ln + pad), padl=padl, padr=int(pad - padl))


def filter_tables_2d(A, lN, res, nm, lD):
    """(filter, kz_phase) of the 2D algorithm as (1, lN) FP64 arrays
    (odtbrain/_alg2d_bpp.py:245-269): the prefactor divided by lN (the
    reference's inverse FFT is normalised) and km*(M-1)."""
    km = (2 * np.pi * nm) / res
    kx = (2 * np.pi * np.fft.fftfreq(lN)).reshape(1, -1)
    dphi0 = 2 * np.pi / A
    klp = (kx ** 2 < km ** 2)
    M = 1. / km * np.sqrt((km ** 2 - kx ** 2) * klp)
    pre = -1j * km / (2 * np.pi)
    pre *= dphi0
    pre *= np.abs(kx) * klp
    pre *= np.exp(-1j * km * (M - 1) * lD)
    filt = np.ascontiguousarray(pre / lN, dtype=np.complex128)
    phase = np.ascontiguousarray(km * (M - 1), dtype=np.float64)
    return filt, phase


def rotation_2d_geometry(angles, ln):
    """Per angle the [m00, m01, m10, m11, off0, off1] that
    ``scipy.ndimage.rotate(image, -angle*180/pi, reshape=False)`` builds
    for an (ln, ln) image (odtbrain/_alg2d_bpp.py:312-321); the angle in
    degrees is formed in the reference's operation order."""
    angles = np.asarray(angles).reshape(-1)
    out = np.empty((angles.size, 6), dtype=np.float64)
    center = (np.asarray((ln, ln)) - 1) / 2
    for i in range(angles.size):
        deg = -angles[i] * 180 / np.pi
        c, s = special.cosdg(deg), special.sindg(deg)
        mat = np.array([[c, s], [-s, c]])
        out[i, :4] = mat.reshape(-1)
        out[i, 4:] = center - mat @ center
    return out
