"""TEST INFRASTRUCTURE ONLY -- CPU oracle for ODTbrain's missing-apple-core
correction ``odtbrain.apple.correct`` (odtbrain/apple.py:8-363).

Only ``tests/``, ``__graft_entry__.smoke()`` and the CPU legs of
``bench.py`` may import this module; the product never calls it.

Restated with NumPy and the reference's own SciPy dependencies
(scipy.ndimage ``distance_transform_edt`` and ``gaussian_filter``, pinned
``scipy>=1.4,<2``); pyFFTW's single-precision 3D c2c transforms
(apple.py:185-197, unnormalised in both directions, FFTW_PRESERVE_INPUT
being FFTW's default for out-of-place c2c) are ``scipy.fft.fftn`` /
``ifftn(norm="forward")`` on complex64 data, which also compute in single
precision.  Pinned by the reference's golden vector
tests/data/apple__test_correct_reproduce.zip and by outputs of the
reference itself (tests/golden/make_golden.py).
"""
import numpy as np
import scipy.fft
import scipy.ndimage as ndi


def apple_core_3d(shape, res, nm):
    """Boolean mask of the missing apple core in unshifted Fourier space,
    the y axis (axis 1) being the axis of symmetry (apple.py:8-53)."""
    km = (2 * np.pi * nm) / res
    lNx, lNy, lNz = shape
    if lNx != lNz:
        raise ValueError("`shape[0]` and `shape[2]` must be identical!")
    fx = np.fft.fftfreq(lNx).reshape(-1, 1, 1)
    fy = np.fft.fftfreq(lNy).reshape(1, -1, 1)
    fz = np.fft.fftfreq(lNz).reshape(1, 1, -1)
    ky = 2 * np.pi * fy
    kxz = 2 * np.pi * np.sqrt(fx ** 2 + fz ** 2)
    kr = 2 * np.pi * np.sqrt(fx ** 2 + fy ** 2 + fz ** 2)
    core = np.zeros(shape, dtype=bool)
    root = 2 * km * kxz - kxz ** 2
    root[root < 0] = 0
    core[np.abs(ky) > np.sqrt(root)] = True
    core[kr > np.sqrt(2) * km] = False
    return core


def spillover_region(shape, shell=0):
    """Voxels outside the inscribed ellipsoid shrunk by ``shell``
    (apple.py:353-363)."""
    x = np.arange(shape[0]).reshape(-1, 1, 1)
    y = np.arange(shape[1]).reshape(1, -1, 1)
    z = np.arange(shape[2]).reshape(1, 1, -1)
    cx, cy, cz = np.array(shape) / 2
    return (((x - cx) / (cx - shell)) ** 2
            + ((y - cy) / (cy - shell)) ** 2
            + ((z - cz) / (cz - shell)) ** 2) > 1


def ellipsoid_shell(shape, width=20):
    """apple.py:281-286."""
    return spillover_region(shape, shell=0) ^ spillover_region(shape,
                                                               shell=width)


def envelope_gauss(ftdata, core):
    """Gaussian-blurred Fourier amplitude with the core filled from the
    axis-swapped volume and then from the nearest known voxel
    (apple.py:289-350)."""
    hull = np.abs(ftdata)
    hull[core] = np.nan
    shx, shy, _ = hull.shape
    maxsh = max(shx, shy)
    dsh = abs(shy - shx) // 2
    if shx > shy:
        sl = (slice(0, shx), slice(dsh, shy + dsh), slice(0, shx))
    else:
        sl = (slice(dsh, shx + dsh), slice(0, shy), slice(dsh, shx + dsh))
    hull_pad = np.zeros((maxsh, maxsh, maxsh), dtype=float)
    hull_pad[sl] = np.fft.fftshift(hull)
    core_pad = np.zeros((maxsh, maxsh, maxsh), dtype=bool)
    core_pad[sl] = np.fft.fftshift(core)
    hull_pad[core_pad] = np.transpose(hull_pad, (1, 0, 2))[core_pad]
    invalid = np.isnan(hull_pad)
    ind = ndi.distance_transform_edt(invalid, return_distances=False,
                                     return_indices=True)
    hull_pad[:] = hull_pad[tuple(ind)]
    hull[:] = np.fft.ifftshift(hull_pad[sl])
    gauss = ndi.gaussian_filter(input=np.fft.fftshift(hull),
                                sigma=np.max(ftdata.shape) / 100,
                                mode="constant", cval=0, truncate=4.0)
    return np.fft.ifftshift(gauss)


def count_to_half(array):
    """apple.py:266-278."""
    num = 0
    for item in array[1:]:
        if item < array[0] / 2:
            break
        num += 1
    return num


def constraint_nn(data, mask=None, bg_shell=None):
    """apple.py:56-72."""
    if np.iscomplexobj(data):
        data.imag[:] = 0
    if bg_shell is not None:
        data.real[bg_shell] = 0
    spov = spillover_region(data.shape)
    data.real[spov] = 0
    lowri = data.real < 0
    if mask is not None:
        lowri *= mask
    data.real[lowri] = 0


def constraint_sh(data, mask=None, bg_shell=None):
    """apple.py:75-110."""
    if np.iscomplexobj(data):
        data.imag[:] = 0
    spov = spillover_region(data.shape)
    if bg_shell is not None:
        spov |= bg_shell
    fmin = np.min(data.real[spov])
    fmax = np.max(data.real[spov])
    full_hist, full_edge = np.histogram(data.real, bins=100,
                                        range=(fmin, fmax))
    de = full_edge[1] - full_edge[0]
    full_f = full_edge[1:] - de / 2
    idx_c = np.argmax(full_hist)
    idx_start = idx_c - count_to_half(full_hist[:idx_c][::-1])
    idx_end = idx_c + count_to_half(full_hist[idx_c:])
    below = (data.real > fmin) * (data.real < full_f[idx_start])
    above = (data.real > full_f[idx_end]) * (data.real < fmax)
    out = below | above
    if mask is not None:
        out *= mask
    data.real[out] *= .5
    if bg_shell is not None:
        data.real[bg_shell] *= .5


def _fft(a):
    return scipy.fft.fftn(a, axes=(0, 1, 2)).astype(np.complex64, copy=False)


def _ifft(a):
    return scipy.fft.ifftn(a, axes=(0, 1, 2), norm="forward") \
        .astype(np.complex64, copy=False)


def correct(f, res, nm, method="nn", mask=None, bg_shell_width=None,
            enforce_envelope=0.95, max_iter=100, min_diff=.01,
            return_iterations=False):
    """The loop of apple.py:113-263 (progress counters left out).
    Returns the complex64 result, and the number of iterations run with
    ``return_iterations``."""
    if enforce_envelope < 0 or enforce_envelope > 1:
        raise ValueError("`enforce_envelope` must be in interval [0, 1]")
    core = apple_core_3d(shape=f.shape, res=res, nm=nm)
    data = np.empty(f.shape, dtype=np.complex64)
    data.real[:] = np.real(f)
    data.imag[:] = 0
    ftdata = _fft(data)
    ftdata_orig = ftdata.copy()
    if enforce_envelope:
        ftevlp = envelope_gauss(ftdata_orig, core)
    init_state = np.sum(np.abs(ftdata_orig[core])) / data.size
    prev_state = init_state
    bg_shell = (ellipsoid_shell(data.shape, width=bg_shell_width)
                if bg_shell_width is not None else None)
    iterations = 0
    for ii in range(max_iter):
        if method == "nn":
            constraint_nn(data=data, mask=mask, bg_shell=bg_shell)
        elif method == "sh":
            constraint_sh(data=data, mask=mask, bg_shell=bg_shell)
        ftdata = _fft(data)
        if enforce_envelope:
            high = np.abs(ftdata) > ftevlp
            ftdata[high] *= enforce_envelope
        if method == "sh":
            ftdata_orig[0, 0, 0] = (ftdata_orig[0, 0, 0] + ftdata[0, 0, 0]) / 2
        ftdata[~core] = ftdata_orig[~core]
        data = _ifft(ftdata)
        data[:] /= data.size
        iterations = ii + 1
        cur_state = np.sum(np.abs(ftdata[core])) / data.size
        cur_diff = cur_state - prev_state
        if ii == 0:
            norm = cur_diff
        else:
            if np.abs(cur_diff / norm) < min_diff:
                break
        prev_state = cur_state
    if return_iterations:
        return data, iterations
    return data
