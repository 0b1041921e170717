"""TEST INFRASTRUCTURE ONLY -- FP64 CPU oracle for ODTbrain's 3D filtered
backpropagation.

This module restates, in NumPy plus the C resampler in ``oracle/spline.c``,
the algorithm of

* ``odtbrain.backpropagate_3d``        (odtbrain/_alg3d_bpp.py:84-555)
* ``odtbrain.backpropagate_3d_tilted`` (odtbrain/_alg3d_bppt.py:374-949)
* ``odtbrain.util.compute_angle_weights_1d`` (odtbrain/util.py:4-67)

in FP64.  It is the checker for the GPU product: only ``tests/``,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` may
import it.  The product never calls it.

Third-party numerics the reference calls, and how they are stood in for:

* FFTW via pyFFTW (pinned ``pyfftw>=0.9.2,<1``): unnormalised forward and
  backward c2c FFTs -> ``scipy.fft`` (pocketfft) with ``norm="forward"`` for
  the backward transform, so both are unnormalised like ``FFTW.execute()``.
* numexpr: ``exp(factor*z)`` -> NumPy.
* scipy.ndimage (pinned ``scipy>=1.4,<2``): spline prefilter and resampling ->
  ``oracle/spline.c`` (restated from the published B-spline algorithms and
  black-box behaviour of scipy 1.18.1; the CPU tests check it against the
  installed scipy).

Pinning: the CPU tests compare this oracle against the reference's own golden
vectors (tests/data/alg3d_bpp__*.zip, re-saved as fixtures under
``tests/golden/``) and against outputs of the unmodified reference generated
by ``tests/golden/make_golden.py``.

Divergence kept on purpose: for ``intp_order`` 0 and 1 the reference's
``_rotate`` (odtbrain/_alg3d_bpp.py:73-81) writes into the array it is
reading, which corrupts the result; this oracle (like the GPU product)
computes the documented out-of-place rotation, which is what
``backpropagate_3d_tilted`` computes for the same inputs.
"""
import ctypes
import os

import numpy as np
import scipy.fft
from scipy import special

from . import build as _build

_LIB = None


def _lib():
    global _LIB
    if _LIB is None:
        path = _build.build()
        lib = ctypes.CDLL(path)
        dp = ctypes.POINTER(ctypes.c_double)
        lib.odto_rotate_y_acc.argtypes = [
            dp, dp, ctypes.c_long, ctypes.c_long, ctypes.c_long, dp, dp,
            ctypes.c_int, ctypes.c_int]
        lib.odto_rotate_y_acc.restype = ctypes.c_int
        lib.odto_affine3d_acc.argtypes = [
            dp, dp, dp, ctypes.c_long, ctypes.c_long, ctypes.c_long, dp, dp,
            ctypes.c_int, ctypes.c_int]
        lib.odto_affine3d_acc.restype = ctypes.c_int
        lib.odto_prefilter_line.argtypes = [dp, ctypes.c_long, ctypes.c_long,
                                            ctypes.c_int]
        lib.odto_prefilter_line.restype = None
        _LIB = lib
    return _LIB


def _ptr(a):
    assert a.dtype == np.float64 and a.flags.c_contiguous
    return a.ctypes.data_as(ctypes.POINTER(ctypes.c_double))


# ------------------------------------------------------------ scipy stand-ins
def rotate_matrix_offset(plane_shape, angle_deg):
    """Matrix and offset ``scipy.ndimage.rotate(reshape=False)`` builds
    (scipy/ndimage/_interpolation.py, ``rotate``: cosdg/sindg, matrix
    [[c, s], [-s, c]], offset = in_center - R @ out_center)."""
    c, s = special.cosdg(angle_deg), special.sindg(angle_deg)
    rot_matrix = np.array([[c, s], [-s, c]])
    shp = np.asarray(plane_shape)
    out_center = rot_matrix @ ((shp - 1) / 2)
    in_center = (shp - 1) / 2
    return rot_matrix, in_center - out_center


def rotate_planes_y(arr, angle_deg, order, nthreads=0, out=None):
    """``scipy.ndimage.rotate(arr, angle_deg, axes=(0, 2), reshape=False,
    order=order, mode="constant", cval=0)`` for a real (z, y, x) volume,
    accumulated into ``out`` (out-of-place; odtbrain/_alg3d_bpp.py:68-81)."""
    arr = np.ascontiguousarray(arr, dtype=np.float64)
    if out is None:
        out = np.zeros_like(arr)
    nz, ny, nx = arr.shape
    mat, off = rotate_matrix_offset((nz, nx), angle_deg)
    mat = np.ascontiguousarray(mat, dtype=np.float64)
    off = np.ascontiguousarray(off, dtype=np.float64)
    rc = _lib().odto_rotate_y_acc(_ptr(arr), _ptr(out), nz, ny, nx,
                                  _ptr(mat), _ptr(off), int(order),
                                  int(nthreads))
    if rc:
        raise ValueError("unsupported spline order %r" % order)
    return out


def affine_transform_3d(arr, matrix, offset, order, nthreads=0, out=None):
    """``scipy.ndimage.affine_transform(arr, matrix, offset, order=order,
    mode="constant", cval=0)`` for a real 3D array, accumulated into
    ``out``."""
    arr = np.ascontiguousarray(arr, dtype=np.float64)
    if out is None:
        out = np.zeros_like(arr)
    work = np.empty_like(arr)
    mat = np.ascontiguousarray(matrix, dtype=np.float64)
    off = np.ascontiguousarray(offset, dtype=np.float64)
    n0, n1, n2 = arr.shape
    rc = _lib().odto_affine3d_acc(_ptr(arr), _ptr(out), _ptr(work), n0, n1,
                                  n2, _ptr(mat), _ptr(off), int(order),
                                  int(nthreads))
    if rc:
        raise ValueError("unsupported spline order %r" % order)
    return out


def spline_filter_line(line, order):
    """Mirror-boundary B-spline prefilter of a 1D real line."""
    c = np.array(line, dtype=np.float64, copy=True)
    _lib().odto_prefilter_line(_ptr(c), c.size, 1, int(order))
    return c


# ------------------------------------------------------------------ util.py
def compute_angle_weights_1d(angles):
    """odtbrain/util.py:4-67: weights proportional to the spacing of the
    neighbouring angles, wrapped modulo pi, duplicates sharing one slot;
    mean 1."""
    angles = np.asarray(angles, dtype=float)
    wrapped = (angles.flatten() - np.min(angles)) % np.pi
    unq, unq_rev, unq_cnt = np.unique(wrapped, return_inverse=True,
                                      return_counts=True)
    order = np.argsort(unq)
    srt = unq[order]
    cnt = unq_cnt[order]
    da = (np.roll(srt, -1) - np.roll(srt, 1)) % np.pi
    total = np.sum(da)
    da /= cnt
    srt_w = da / total * wrapped.size
    unq_w = np.zeros_like(srt_w)
    unq_w[order] = srt_w
    return unq_w[unq_rev]


# ------------------------------------------------------------ common filter
def padding_geometry(lny, lnx, padding, padfac):
    """odtbrain/_alg3d_bpp.py:285-304."""
    if padding[0]:
        orderx = int(max(64., 2 ** np.ceil(np.log(lnx * padfac) / np.log(2))))
        padx = orderx - lnx
    else:
        padx = 0
    if padding[1]:
        ordery = int(max(64., 2 ** np.ceil(np.log(lny * padfac) / np.log(2))))
        pady = ordery - lny
    else:
        pady = 0
    padyl = int(np.ceil(pady / 2))
    padxl = int(np.ceil(padx / 2))
    return dict(padx=padx, pady=pady, padyl=padyl, padyr=pady - padyl,
                padxl=padxl, padxr=padx - padxl, lNx=lnx + padx,
                lNy=lny + pady)


def pad_projection(proj, geo, padding, padval):
    """odtbrain/_alg3d_bpp.py:493-506 (np.pad edge / linear_ramp / none)."""
    if not (padding[0] and padding[1]):
        return np.array(proj, dtype=np.complex128)
    width = ((geo["padyl"], geo["padyr"]), (geo["padxl"], geo["padxr"]))
    if isinstance(padval, str) and padval == "edge":
        return np.pad(proj, width, mode="edge")
    return np.pad(proj, width, mode="linear_ramp", end_values=(padval,))


def filter_constants(A, lNx, lNy, res, nm, lD):
    """odtbrain/_alg3d_bpp.py:317, 371-399 (and _alg3d_bppt.py:737-771)."""
    km = (2 * np.pi * nm) / res
    kx = (2 * np.pi * np.fft.fftfreq(lNx)).reshape(1, -1)
    ky = (2 * np.pi * np.fft.fftfreq(lNy)).reshape(-1, 1)
    dphi0 = 2 * np.pi / A
    klp = (kx ** 2 + ky ** 2 < km ** 2)
    M = 1. / km * np.sqrt((km ** 2 - kx ** 2 - ky ** 2) * klp)
    prefactor = -1j * km / (2 * np.pi)
    prefactor *= dphi0
    return dict(km=km, kx=kx, ky=ky, klp=klp, M=M, prefactor=prefactor)


_TABLE_LIMIT = 2 << 30


def propagator_table(f2_exp_fac, zv, cache=None):
    """``filter2 = exp(factor*z)`` for every plane (odtbrain/_alg3d_bpp.py:
    429-437, the default ``save_memory=False`` path), or None when it would
    exceed 2 GiB.  ``cache`` (a dict) keeps the table across calls."""
    nbytes = zv.shape[0] * f2_exp_fac.size * 16
    if nbytes > _TABLE_LIMIT:
        return None
    key = (f2_exp_fac.shape, zv.shape[0], f2_exp_fac.tobytes()[:4096],
           float(np.abs(f2_exp_fac).sum()))
    if cache is not None and cache.get("key") == key:
        return cache["table"]
    table = np.exp(f2_exp_fac[None, :, :] * zv)
    if cache is not None:
        cache["key"] = key
        cache["table"] = table
    return table


def _filtered_slab(spec, f2_exp_fac, zv, geo, lny, lnx, fft_workers,
                   zchunk=16, table=None):
    """Propagate one filtered spectrum to every z plane and crop
    (odtbrain/_alg3d_bpp.py:514-528): unnormalised backward FFT of
    ``exp(factor*z_p) * spectrum`` for each plane p."""
    lNz = zv.shape[0]
    out = np.empty((lNz, lny, lnx), dtype=np.complex128)
    ys = slice(geo["padyl"], geo["padyl"] + lny)
    xs = slice(geo["padxl"], geo["padxl"] + lnx)
    for p0 in range(0, lNz, zchunk):
        p1 = min(lNz, p0 + zchunk)
        if table is not None:
            filt = table[p0:p1]
        else:
            filt = np.exp(f2_exp_fac[None, :, :] * zv[p0:p1])
        inarr = filt * spec[None, :, :]
        res = scipy.fft.ifftn(inarr, axes=(1, 2), norm="forward",
                              workers=fft_workers)
        out[p0:p1] = res[:, ys, xs]
    return out


def _prepare(uSin, angles, res, nm, lD, padding, padfac, weights):
    uSin = np.array(uSin, dtype=np.complex128, copy=True)
    A = uSin.shape[0]
    lny, lnx = uSin.shape[1], uSin.shape[2]
    geo = padding_geometry(lny, lnx, padding, padfac)
    if weights is not None:
        uSin *= np.asarray(weights).reshape(-1, 1, 1)
    fc = filter_constants(A, geo["lNx"], geo["lNy"], res, nm, lD)
    lNz = lnx
    center = lNz / 2.0
    z = np.linspace(-center, center, lNz, endpoint=False)
    zv = z.reshape(-1, 1, 1)
    f2_exp_fac = 1j * fc["km"] * (fc["M"] - 1)
    return uSin, geo, fc, zv, f2_exp_fac


def backpropagate_3d(uSin, angles, res, nm, lD=0, weight_angles=True,
                     onlyreal=False, padding=(True, True), padfac=1.75,
                     padval="edge", intp_order=2, nthreads=0,
                     fft_workers=None, angle_subset=None, cache=None):
    """FP64 restatement of ``odtbrain.backpropagate_3d``
    (odtbrain/_alg3d_bpp.py:84-555), out-of-place rotation.

    Returns a complex128 volume of shape (Nx, Ny, Nx) indexed [z, y, x]
    (float64 when ``onlyreal``).  ``angle_subset`` restricts the sum to some
    angle indices (used for bounded CPU-baseline timing); the filter
    constants still use the full angle count, as the reference does.
    """
    angles = np.asarray(angles)
    A = angles.size
    weights = (compute_angle_weights_1d(angles) if weight_angles else None)
    uSin, geo, fc, zv, f2 = _prepare(uSin, angles, res, nm, lD, padding,
                                     padfac, weights)
    lny, lnx = uSin.shape[1], uSin.shape[2]
    lNx, lNy = geo["lNx"], geo["lNy"]
    prefactor = fc["prefactor"] * np.abs(fc["kx"]) * fc["klp"]
    prefactor = prefactor * np.exp(-1j * fc["km"] * (fc["M"] - 1) * lD)
    out_re = np.zeros((lnx, lny, lnx))
    out_im = None if onlyreal else np.zeros((lnx, lny, lnx))
    idx = range(A) if angle_subset is None else angle_subset
    table = propagator_table(f2, zv, cache)
    for aa in idx:
        oneslice = pad_projection(uSin[aa], geo, padding, padval)
        spec = scipy.fft.fftn(oneslice, axes=(0, 1), workers=fft_workers)
        spec *= prefactor / (lNx * lNy)
        slab = _filtered_slab(spec, f2, zv, geo, lny, lnx, fft_workers,
                              table=table)
        phi0 = np.rad2deg(angles[aa])
        rotate_planes_y(slab.real, -phi0, intp_order, nthreads, out=out_re)
        if not onlyreal:
            rotate_planes_y(slab.imag, -phi0, intp_order, nthreads,
                            out=out_im)
    if onlyreal:
        return out_re
    return out_re + 1j * out_im


# ------------------------------------------------------- tilted geometry
def norm_vec(vector):
    """odtbrain/_alg3d_bppt.py:26-30."""
    v = np.array(vector)
    return v / np.sqrt(np.sum(v ** 2))


def sphere_points_from_angles_and_tilt(angles, tilted_axis):
    """odtbrain/_alg3d_bppt.py:230-371."""
    tilted_axis = norm_vec(tilted_axis)
    u, v, w = tilted_axis
    newang = np.zeros((angles.shape[0], 3), dtype=float)
    newang[:, 0] = np.sin(angles - angles[0])
    newang[:, 2] = np.cos(angles - angles[0])
    theta = np.arccos(v)
    if np.allclose(u, 0) and np.allclose(w, 0):
        phi = 0
    else:
        phi = np.arctan2(u, w)
    newang *= np.cos(theta)
    Rx = np.array([[1, 0, 0],
                   [0, np.cos(theta), -np.sin(theta)],
                   [0, np.sin(theta), np.cos(theta)]])
    for ii in range(newang.shape[0]):
        newang[ii] = np.dot(Rx, newang[ii])
    newang = newang - (newang[0] - np.array([0, 0, 1])).reshape(1, 3)
    Ry = np.array([[+np.cos(phi), 0, np.sin(phi)],
                   [0, 1, 0],
                   [-np.sin(phi), 0, np.cos(phi)]])
    for jj in range(newang.shape[0]):
        newang[jj] = np.dot(Ry, newang[jj])
    return newang


def rotate_points_to_axis(points, axis):
    """odtbrain/_alg3d_bppt.py:33-120."""
    axis = norm_vec(axis)
    u, v, w = axis
    points = np.array(points)
    phi = np.arctan2(u, w)
    theta = np.arccos(v)
    Rphi = np.array([[np.cos(phi), 0, -np.sin(phi)],
                     [0, 1, 0],
                     [np.sin(phi), 0, np.cos(phi)]])
    Rtheta = np.array([[1, 0, 0],
                       [0, np.cos(theta), np.sin(theta)],
                       [0, -np.sin(theta), np.cos(theta)]])
    DR1 = np.dot(Rtheta, Rphi)
    DR = np.dot(Rphi.T, DR1)
    rotpoints = np.zeros((len(points), 3))
    for ii, pnt in enumerate(points):
        rotpoints[ii] = np.dot(DR, pnt)
    return rotpoints


def rotation_matrix_from_point(point, ret_inv=False):
    """odtbrain/_alg3d_bppt.py:123-175."""
    x, y, z = point
    phi = np.arctan2(x, z)
    theta = -np.arctan2(y, np.sqrt(x ** 2 + z ** 2))
    Rtheta = np.array([[1, 0, 0],
                       [0, np.cos(theta), -np.sin(theta)],
                       [0, np.sin(theta), np.cos(theta)]])
    Rphi = np.array([[np.cos(phi), 0, -np.sin(phi)],
                     [0, 1, 0],
                     [np.sin(phi), 0, np.cos(phi)]])
    D = np.dot(Rphi, Rtheta)
    Dinv = np.dot(Rtheta.T, Rphi.T)
    if ret_inv:
        return D, Dinv
    return D


def rotation_matrix_from_point_planerot(point, plane_angle, ret_inv=False):
    """odtbrain/_alg3d_bppt.py:178-227."""
    D, Dinv = rotation_matrix_from_point(point, ret_inv=True)
    angz = plane_angle
    Rz = np.array([[np.cos(angz), -np.sin(angz), 0],
                   [np.sin(angz), np.cos(angz), 0],
                   [0, 0, 1]])
    DR = np.dot(D, Rz)
    DRinv = np.dot(Rz.T, Dinv)
    if ret_inv:
        return DR, DRinv
    return DR


def tilted_geometry(angles, tilted_axis, weight_angles, shape_xyz):
    """Host FP64 geometry of odtbrain/_alg3d_bppt.py:644-676, 863, 907-919.

    Returns (weights or None, list of (drotinv, offset) per angle,
    normalised tilted axis)."""
    angles = np.array(angles, copy=True)
    angles = np.squeeze(angles)
    tilted_axis = norm_vec(tilted_axis)
    angz = np.arctan2(tilted_axis[0], tilted_axis[1])
    rotmat = np.array([[np.cos(angz), -np.sin(angz), 0],
                       [np.sin(angz), np.cos(angz), 0],
                       [0, 0, 1]])
    tilted_axis_yz = norm_vec(np.dot(rotmat, tilted_axis))
    weights = None
    if len(angles.shape) == 1:
        if weight_angles:
            weights = compute_angle_weights_1d(angles)
        angles = sphere_points_from_angles_and_tilt(angles, tilted_axis_yz)
    else:
        if weight_angles:
            weights = np.ones(angles.shape[0])
        for ii in range(angles.shape[0]):
            angles[ii] = norm_vec(np.dot(rotmat, angles[ii]))
    points = rotate_points_to_axis(points=angles, axis=tilted_axis_yz)
    c = 0.5 * np.array(shape_xyz) - .5
    mats = []
    for aa in range(points.shape[0]):
        _d, drotinv = rotation_matrix_from_point_planerot(
            points[aa], plane_angle=angz, ret_inv=True)
        offset = c - np.dot(drotinv, c)
        mats.append((drotinv, offset))
    return weights, mats, tilted_axis


def backpropagate_3d_tilted(uSin, angles, res, nm, lD=0,
                            tilted_axis=(0, 1, 0), weight_angles=True,
                            onlyreal=False, padding=(True, True),
                            padfac=1.75, padval="edge", intp_order=2,
                            nthreads=0, fft_workers=None,
                            angle_subset=None, cache=None):
    """FP64 restatement of ``odtbrain.backpropagate_3d_tilted``
    (odtbrain/_alg3d_bppt.py:374-949)."""
    angles = np.asarray(angles)
    A = angles.shape[0]
    lny, lnx = uSin.shape[1], uSin.shape[2]
    shape_xyz = (lnx, lny, lnx)
    weights, mats, taxis = tilted_geometry(angles, tilted_axis,
                                           weight_angles, shape_xyz)
    uSin, geo, fc, zv, f2 = _prepare(uSin, angles, res, nm, lD, padding,
                                     padfac, weights)
    lNx, lNy = geo["lNx"], geo["lNy"]
    u, v, _w = taxis
    filterabs = np.abs(fc["kx"] * v + fc["ky"] * u) * fc["klp"]
    prefactor = fc["prefactor"] * np.exp(-1j * fc["km"] * (fc["M"] - 1) * lD)
    acc_re = np.zeros(shape_xyz)
    acc_im = None if onlyreal else np.zeros(shape_xyz)
    idx = range(A) if angle_subset is None else angle_subset
    table = propagator_table(f2, zv, cache)
    for aa in idx:
        oneslice = pad_projection(uSin[aa], geo, padding, padval)
        spec = scipy.fft.fftn(oneslice, axes=(0, 1), workers=fft_workers)
        spec *= filterabs * prefactor / (lNx * lNy)
        slab = _filtered_slab(spec, f2, zv, geo, lny, lnx, fft_workers,
                              table=table)
        fil_p_t = slab.transpose(2, 1, 0)[:, ::-1, :]
        drotinv, offset = mats[aa]
        affine_transform_3d(fil_p_t.real, drotinv, offset, intp_order,
                            nthreads, out=acc_re)
        if not onlyreal:
            affine_transform_3d(fil_p_t.imag, drotinv, offset, intp_order,
                                nthreads, out=acc_im)
    out_re = acc_re.transpose(2, 1, 0)[:, ::-1, :]
    if onlyreal:
        return np.ascontiguousarray(out_re)
    return np.ascontiguousarray(out_re + 1j *
                                acc_im.transpose(2, 1, 0)[:, ::-1, :])


# ------------------------------------------------------------------ 2D path
def backpropagate_2d(uSin, angles, res, nm, lD=0, weight_angles=True,
                     onlyreal=False, padding=True, padval=0):
    """FP64 restatement of ``odtbrain.backpropagate_2d``
    (odtbrain/_alg2d_bpp.py:134-326): weight, pad along x (2.1x rule,
    linear ramp to ``padval`` or edge values), FFT, filter, per-row
    propagator exp(i km (M-1) yv) with yv = k - ln/2 + 0.5 and normalised
    inverse FFT, crop to (ln, ln), rotate by -phi with scipy.ndimage's
    cubic spline, sum."""
    import scipy.ndimage
    uSin = np.asarray(uSin)
    angles = np.asarray(angles).reshape(-1)
    A, ln = uSin.shape
    sino = uSin * compute_angle_weights_1d(angles)[:, None] if weight_angles \
        else np.array(uSin, dtype=complex)
    lN = int(max(64., 2 ** np.ceil(np.log(ln * 2.1) / np.log(2)))) \
        if padding else ln
    pad = lN - ln
    padl = int(np.ceil(pad / 2))
    widths = ((0, 0), (padl, pad - padl))
    if padval is None:
        sino = np.pad(sino, widths, mode="edge")
    else:
        sino = np.pad(sino, widths, mode="linear_ramp", end_values=(padval,))
    km = (2 * np.pi * nm) / res
    kx = 2 * np.pi * np.fft.fftfreq(lN)
    inside = kx ** 2 < km ** 2
    M = np.sqrt((km ** 2 - kx ** 2) * inside) / km
    pref = (-1j * km / (2 * np.pi)) * (2 * np.pi / A) * np.abs(kx) * inside
    pref = pref * np.exp(-1j * km * (M - 1) * lD)
    spec = scipy.fft.fft(sino, axis=-1) * pref                 # (A, lN)
    yv = np.arange(ln) - ln / 2.0 + 0.5
    prop = np.exp(1j * yv[:, None] * km * (M - 1)[None, :])    # (ln, lN)
    out = np.zeros((ln, ln), dtype=float if onlyreal else complex)
    for i in range(A):
        img = scipy.fft.ifft(spec[i][None, :] * prop, axis=-1)[:, padl:padl + ln]
        deg = -angles[i] * 180 / np.pi
        out += scipy.ndimage.rotate(img.real, deg, reshape=False,
                                    mode="constant", cval=0)
        if not onlyreal:
            out += 1j * scipy.ndimage.rotate(img.imag, deg, reshape=False,
                                             mode="constant", cval=0)
    return out


def odt_to_ri(f, res, nm):
    """FP64 restatement of ``odtbrain.odt_to_ri``
    (odtbrain/_translate_ri.py:5-57): nm * sqrt(f / km^2 + 1), principal
    root, real part made non-negative."""
    km = (2 * np.pi * nm) / res
    ri = nm * np.sqrt(np.asarray(f, dtype=complex) / km ** 2 + 1)
    neg = ri.real < 0
    ri[neg] *= -1
    return ri


def opt_to_ri(f, res, nm):
    """FP64 restatement of ``odtbrain.opt_to_ri``
    (odtbrain/_translate_ri.py:60-93): nm + f * res / (2 pi)."""
    return nm + np.asarray(f) / (2 * np.pi) * res
