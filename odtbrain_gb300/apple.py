"""Drop-in missing-apple-core correction (odtbrain/apple.py).

``correct`` (odtbrain/apple.py:113-263) runs on the GPU
(``odt_apple_correct`` of the C ABI): the volume stays in HBM as complex64,
the 3D FFTs are single precision and unnormalised like the reference's
pyFFTW plans, the constraints, the envelope suppression and the spectrum
restore are fused into the FFT passes, and the stopping test is evaluated
on the device in float32 like the reference's NumPy scalars.  The masks
``apple_core_3d``, ``spillover_region`` and ``ellipsoid_shell`` come from
the same GPU kernel (``odt_apple_flags``).  ``constraint_nn``,
``constraint_sh`` (apple.py:56-110) and ``envelope_gauss`` (:289-350)
called on their own run on the GPU too (``odt_apple_constrain``,
``odt_apple_envelope``), with the kernels ``correct`` uses.

NumPy input gives NumPy output; torch tensors give CUDA tensors.  There is
no CPU fallback.
"""
import ctypes

import numpy as np

from . import _native
from ._alg3d import _device_for, _is_tensor, _to_host, _torch

_METHODS = {"nn": _native.ODT_APPLE_NN, "sh": _native.ODT_APPLE_SH}


def _gauss_weights(shape):
    """The 1D kernel of scipy.ndimage.gaussian_filter for sigma =
    max(shape) / 100, truncate 4 (odtbrain/apple.py:343-347), computed the
    way scipy computes it (FP64, normalised to sum 1)."""
    sigma = float(np.max(shape) / 100)
    radius = int(4.0 * sigma + 0.5)
    x = np.arange(-radius, radius + 1)
    phi = np.exp(-0.5 / (sigma * sigma) * x ** 2)
    return np.ascontiguousarray(phi / phi.sum()), radius


def _desc(shape, res, nm, method="nn", bg_shell_width=None,
          enforce_envelope=0.95, max_iter=100, min_diff=.01):
    d = _native.AppleDesc()
    d.n0, d.n1, d.n2 = (int(v) for v in shape)
    d.res, d.nm = float(res), float(nm)
    d.method = _METHODS.get(method, _native.ODT_APPLE_NONE)
    d.enforce_envelope = float(enforce_envelope)
    d.max_iter = int(max_iter)
    d.min_diff = float(min_diff)
    d.use_bg_shell = int(bg_shell_width is not None)
    d.bg_shell_width = float(bg_shell_width) if bg_shell_width is not None \
        else 0.0
    w, r = _gauss_weights(shape)
    d.gauss_radius = r
    d._weights = w  # keep alive
    d.gauss_weights = w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    return d


def _flags(shape, res=1.0, nm=1.0, bg_shell_width=None, device=None):
    torch = _torch()
    if len(shape) != 3:
        raise ValueError("shape must have three entries")
    if shape[0] != shape[2]:
        raise ValueError("`shape[0]` and `shape[2]` must be identical!")
    dev = device or torch.device("cuda", torch.cuda.current_device())
    d = _desc(shape, res, nm, bg_shell_width=bg_shell_width)
    L = _native.lib()
    with torch.cuda.device(dev):
        fl = torch.empty(tuple(int(v) for v in shape), dtype=torch.uint8,
                         device=dev)
        nb = ctypes.c_uint64()
        _native.check(L.odt_apple_flags_workspace_size(ctypes.byref(d),
                                                       ctypes.byref(nb)))
        ws = torch.empty(nb.value, dtype=torch.uint8, device=dev)
        stream = torch.cuda.current_stream(dev)
        _native.check(L.odt_apple_flags(
            ctypes.byref(d), None, ctypes.c_void_p(fl.data_ptr()),
            ctypes.c_void_p(ws.data_ptr()),
            ctypes.c_void_p(stream.cuda_stream)))
        return fl.cpu().numpy()


def apple_core_3d(shape, res, nm):
    """Boolean mask of the apple core in unshifted Fourier space, the y axis
    being the axis of symmetry (odtbrain/apple.py:8-53)."""
    return (_flags(shape, res, nm) & 1).astype(bool)


def spillover_region(shape, shell=0):
    """Voxels outside the inscribed ellipsoid (odtbrain/apple.py:353-363);
    ``shell`` > 0 shrinks the ellipsoid (shape[0] must equal shape[2])."""
    if shell == 0:
        return (_flags(shape) & 2).astype(bool)
    outer = (_flags(shape) & 2).astype(bool)
    band = (_flags(shape, bg_shell_width=shell) & 4).astype(bool)
    return outer ^ band


def ellipsoid_shell(shape, width=20):
    """Background ellipsoid shell (odtbrain/apple.py:281-286)."""
    return (_flags(shape, bg_shell_width=width) & 4).astype(bool)


def _voxel_bytes(m, shape, dev):
    """A boolean array (NumPy or torch, broadcast to `shape`) as device
    bytes, 1 where it is nonzero."""
    torch = _torch()
    if _is_tensor(m):
        return (m.to(dev) != 0).expand(shape).to(torch.uint8).contiguous()
    return torch.from_numpy(np.ascontiguousarray(
        np.broadcast_to(np.asarray(m) != 0, shape), dtype=np.uint8)).to(dev)


def _real_bits(dtype):
    """32 or 64 for a float / complex NumPy or torch dtype, else None."""
    torch = _torch()
    if isinstance(dtype, torch.dtype):
        return {torch.float32: 32, torch.complex64: 32, torch.float64: 64,
                torch.complex128: 64}.get(dtype)
    return {np.dtype(np.float32): 32, np.dtype(np.complex64): 32,
            np.dtype(np.float64): 64,
            np.dtype(np.complex128): 64}.get(np.dtype(dtype))


def _constrain(data, mask, bg_shell, method):
    """One constraint of apple.py:56-110 in place on the GPU
    (``odt_apple_constrain``): NumPy arrays are copied to the device and
    back, CUDA tensors are changed where they lie."""
    torch = _torch()
    shape = tuple(data.shape)
    if len(shape) != 3:
        raise ValueError("`data` must be a 3D array")
    bits = _real_bits(data.dtype)
    if bits is None:
        raise TypeError("`data` must be float32, float64, complex64 or "
                        "complex128, not {}".format(data.dtype))
    is_t = _is_tensor(data)
    dev = _device_for(data)
    d = _native.AppleDesc()
    d.n0, d.n1, d.n2 = (int(v) for v in shape)
    d.method = method
    L = _native.lib()
    with torch.cuda.device(dev):
        if is_t and data.is_cuda and data.is_contiguous():
            t = data
        elif is_t:
            t = data.to(dev).contiguous()
        else:
            t = torch.from_numpy(np.ascontiguousarray(data)).to(dev)
        mk = _voxel_bytes(mask, shape, dev) if mask is not None else None
        sh = _voxel_bytes(bg_shell, shape, dev) if bg_shell is not None \
            else None
        nb = ctypes.c_uint64()
        _native.check(L.odt_apple_constrain_workspace_size(ctypes.byref(d),
                                                           ctypes.byref(nb)))
        ws = torch.empty(nb.value, dtype=torch.uint8, device=dev)
        stream = torch.cuda.current_stream(dev)
        _native.check(L.odt_apple_constrain(
            ctypes.byref(d), bits, int(t.is_complex()),
            ctypes.c_void_p(t.data_ptr()),
            ctypes.c_void_p(mk.data_ptr() if mk is not None else 0),
            ctypes.c_void_p(sh.data_ptr() if sh is not None else 0),
            ctypes.c_void_p(ws.data_ptr()), nb.value,
            ctypes.c_void_p(stream.cuda_stream)))
        if t is data:
            return
        if is_t:
            data.copy_(t)
        else:
            data[...] = _to_host(t)


def constraint_nn(data, mask=None, bg_shell=None):
    """Non-negativity constraint, in place (drop-in for
    ``odtbrain.apple.constraint_nn``, odtbrain/apple.py:56-72): the
    imaginary part set to 0; the real part set to 0 in ``bg_shell``,
    outside the inscribed ellipsoid and where it is negative (where
    ``mask`` is set, if given)."""
    _constrain(data, mask, bg_shell, _native.ODT_APPLE_NN)


def constraint_sh(data, mask=None, bg_shell=None):
    """Symmetric-histogram background constraint, in place (drop-in for
    ``odtbrain.apple.constraint_sh``, odtbrain/apple.py:75-110): the real
    values outside the half-maximum band of the histogram over
    [min, max] of the background region halved (where ``mask`` is set, if
    given), ``bg_shell`` halved, the imaginary part set to 0.  Histogram
    arithmetic in the data's precision like the reference's NumPy code."""
    _constrain(data, mask, bg_shell, _native.ODT_APPLE_SH)


def envelope_gauss(ftdata, core):
    """Gaussian-filtered envelope of the Fourier amplitude without the
    apple core (drop-in for ``odtbrain.apple.envelope_gauss``,
    odtbrain/apple.py:289-350), on the GPU (``odt_apple_envelope``).

    ``ftdata``: spectrum in FFT order, shape (N, M, N); ``core``: boolean
    mask of the same shape.  The result has the real type of ``ftdata``
    (float32 for complex64 / float32 input, float64 otherwise), NumPy for
    NumPy input and a CUDA tensor for a tensor."""
    torch = _torch()
    shape = tuple(ftdata.shape)
    if len(shape) != 3:
        raise ValueError("`ftdata` must be a 3D array")
    if shape[0] != shape[2]:
        raise ValueError("`shape[0]` and `shape[2]` must be identical!")
    is_t = _is_tensor(ftdata)
    dev = _device_for(ftdata)
    bits = _real_bits(ftdata.dtype) or 64
    cdt = torch.complex64 if bits == 32 else torch.complex128
    d = _native.AppleDesc()
    d.n0, d.n1, d.n2 = (int(v) for v in shape)
    w, r = _gauss_weights(shape)
    d.gauss_radius = r
    d.gauss_weights = w.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    L = _native.lib()
    with torch.cuda.device(dev):
        if is_t:
            t = ftdata.to(dev)
        else:
            t = torch.from_numpy(np.ascontiguousarray(ftdata)).to(dev)
        t = t.to(cdt).contiguous()
        cb = _voxel_bytes(core, shape, dev)
        out = torch.empty(shape, device=dev,
                          dtype=torch.float32 if bits == 32
                          else torch.float64)
        nb = ctypes.c_uint64()
        _native.check(L.odt_apple_envelope_workspace_size(ctypes.byref(d),
                                                          ctypes.byref(nb)))
        ws = torch.empty(nb.value, dtype=torch.uint8, device=dev)
        stream = torch.cuda.current_stream(dev)
        _native.check(L.odt_apple_envelope(
            ctypes.byref(d), bits, ctypes.c_void_p(t.data_ptr()),
            ctypes.c_void_p(cb.data_ptr()), ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(ws.data_ptr()), nb.value,
            ctypes.c_void_p(stream.cuda_stream)))
    if is_t:
        return out
    return _to_host(out)


def count_to_half(array):
    """First index at which the values drop below half of ``array[0]``
    (odtbrain/apple.py:266-278)."""
    num = 0
    for item in array[1:]:
        if item < array[0] / 2:
            break
        num += 1
    return num


def correct(f, res, nm, method="nn", mask=None, bg_shell_width=None,
            enforce_envelope=0.95, max_iter=100, min_diff=.01,
            count=None, max_count=None):
    r"""Fill the missing apple core of the object function (drop-in for
    ``odtbrain.apple.correct``, odtbrain/apple.py:113-263).

    Same parameters, validation, progress counters and result (complex64,
    the real part of ``f`` corrected) as the reference."""
    if enforce_envelope < 0 or enforce_envelope > 1:
        raise ValueError("`enforce_envelope` must be in interval [0, 1]")
    if max_count is not None:
        with max_count.get_lock():
            max_count.value += max_iter + 2
    torch = _torch()
    shape = tuple(f.shape)
    if len(shape) != 3:
        raise ValueError("`f` must be a 3D array")
    if shape[0] != shape[2]:
        raise ValueError("`shape[0]` and `shape[2]` must be identical!")
    is_t = _is_tensor(f)
    dev = _device_for(f)
    d = _desc(shape, res, nm, method, bg_shell_width, enforce_envelope,
              max_iter, min_diff)
    L = _native.lib()
    with torch.cuda.device(dev):
        if is_t:
            t = f.to(dev)
        elif np.asarray(f).dtype.kind in "fc":
            # the array as it is (a plain copy, fast from pinned memory);
            # the real part is taken on the device
            t = torch.from_numpy(np.ascontiguousarray(np.asarray(f))).to(dev)
        else:
            t = torch.from_numpy(np.ascontiguousarray(
                np.real(np.asarray(f)), dtype=np.float32)).to(dev)
        fr = (t.real if t.is_complex() else t).to(torch.float32).contiguous()
        mk = None
        if mask is not None:
            m = mask.to(dev) if _is_tensor(mask) else torch.from_numpy(
                np.array(np.broadcast_to(np.asarray(mask), shape),
                         dtype=np.uint8)).to(dev)
            mk = m.expand(shape).to(torch.uint8).contiguous()
        ws_bytes = ctypes.c_uint64()
        _native.check(L.odt_apple_workspace_size(ctypes.byref(d),
                                                 ctypes.byref(ws_bytes)))
        ws = torch.empty(max(ws_bytes.value, 1), dtype=torch.uint8,
                         device=dev)
        out = torch.empty(shape, dtype=torch.complex64, device=dev)
        if count is not None:
            with count.get_lock():
                count.value += 1
        iters = ctypes.c_int32(0)
        stream = torch.cuda.current_stream(dev)
        _native.check(L.odt_apple_correct(
            ctypes.byref(d), ctypes.c_void_p(fr.data_ptr()),
            ctypes.c_void_p(mk.data_ptr() if mk is not None else 0),
            ctypes.c_void_p(out.data_ptr()), ctypes.c_void_p(ws.data_ptr()),
            ws_bytes.value, ctypes.byref(iters),
            ctypes.c_void_p(stream.cuda_stream)))
    if count is not None:
        if max_iter == 0:
            # the reference reads its loop variable after an empty loop
            raise UnboundLocalError("cannot access local variable 'ii' where "
                                    "it is not associated with a value")
        with count.get_lock():
            count.value += 1 + iters.value + (max_iter - iters.value)
    if is_t:
        return out
    return _to_host(out)
