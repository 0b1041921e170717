"""Drop-in ``backpropagate_3d`` and ``backpropagate_3d_tilted``.

Same signatures, validation, errors, progress counters, ``copy`` semantics
and output layout as the reference (odtbrain/_alg3d_bpp.py:84-555 and
odtbrain/_alg3d_bppt.py:374-949).  The host computes the FP64 constants; the
per-angle filtering, propagation, resampling and accumulation run on the GPU
through the C ABI of ``libodtbrain_gb300.so``.  The GPU arithmetic is FP32
(compensated accumulation across angles); the result is returned in the
precision ``dtype`` asks for.

Inputs may be NumPy arrays (the result is a NumPy array) or torch tensors
(the result is a CUDA tensor on the same device, or on the current CUDA
device for CPU tensors).

:class:`Backprop3D` is the prepared form: geometry, plan, workspace and
output buffers built once, then applied to device-resident sinograms.
"""
import collections
import ctypes
import multiprocessing as mp
import threading
import warnings

import numpy as np

from . import _geometry as geom
from . import _native

ncores = mp.cpu_count()

# workspace the plan may use; save_memory trades batch size for memory
_WS_DEFAULT = 16 << 30
_WS_SAVE_MEMORY = 1 << 30

_PLAN_CACHE = collections.OrderedDict()
_PLAN_CACHE_SIZE = 8
_PLAN_LOCK = threading.Lock()

# device copies of the FP64 per-angle tables (weights, geometry): building
# the rotation geometry of 200 angles takes ~0.75 ms on the host, so repeated
# calls with the same angles reuse them
_TABLE_CACHE = collections.OrderedDict()
_TABLE_CACHE_SIZE = 8


def _torch():
    import torch
    return torch


def _is_tensor(x):
    try:
        torch = _torch()
    except ImportError:  # pragma: no cover
        return False
    return isinstance(x, torch.Tensor)


def _validate_common(uSin_shape, A, padding, coords, num_cores, dtype):
    """odtbrain/_alg3d_bpp.py:237-264 (same messages and exception types)."""
    if len(uSin_shape) != 3:
        raise ValueError("Input data `uSin` must have shape (A,Ny,Nx).")
    if uSin_shape[0] != A:
        raise ValueError("`len(angles)` must be  equal to `len(uSin)`.")
    if len(list(padding)) != 2:
        raise ValueError("`padding` must be boolean tuple of length 2!")
    if np.array(padding).dtype is not np.dtype(bool):
        raise ValueError("Parameter `padding` must be boolean tuple.")
    if coords is not None:
        raise NotImplementedError("Setting coordinates is not yet supported.")
    if num_cores > ncores:
        raise ValueError("`num_cores` must not exceed number "
                         + "of physical cores: {}".format(ncores))
    if dtype is None:
        dtype = np.float64
    dtype = np.dtype(dtype)
    if dtype.name not in ["float32", "float64"]:
        raise ValueError("dtype must be float32 or float64!")
    return dtype


def _pad_mode(padding, padval):
    if not (padding[0] and padding[1]):
        if padding[0] or padding[1]:
            # the reference builds mismatched filter and data shapes here
            # and fails with a NumPy broadcast ValueError
            raise ValueError("operands could not be broadcast together: "
                             "padding must be (True, True) or "
                             "(False, False)")
        return _native.ODT_PAD_NONE, 0j
    if isinstance(padval, str):
        if padval != "edge":
            raise ValueError("`padval` must be 'edge' or a number")
        return _native.ODT_PAD_EDGE, 0j
    return _native.ODT_PAD_RAMP, complex(padval)


def _get_tables(key, build):
    """(weights, geometry, taxis) for `key`: `build()` returns the host
    weights (or None), the geometry and the tilted axis; the device tensors
    are cached and must not be modified."""
    with _PLAN_LOCK:
        hit = _TABLE_CACHE.get(key)
        if hit is not None:
            _TABLE_CACHE.move_to_end(key)
            return hit
    torch = _torch()
    device = torch.device("cuda", key[0])
    weights, geometry, taxis = build()
    dw = (torch.from_numpy(np.ascontiguousarray(weights, dtype=np.float64))
          .to(device) if weights is not None else None)
    dg = torch.from_numpy(np.ascontiguousarray(geometry, dtype=np.float64)) \
        .to(device)
    hit = (dw, dg, taxis)
    with _PLAN_LOCK:
        _TABLE_CACHE[key] = hit
        while len(_TABLE_CACHE) > _TABLE_CACHE_SIZE:
            _TABLE_CACHE.popitem(last=False)
    return hit


def _get_plan(key, build_desc):
    """The cached native plan for `key` (built by `build_desc` on a miss).
    Instances with equal keys share one plan, and so its device status
    word: status reporting is per plan, not per instance."""
    with _PLAN_LOCK:
        plan = _PLAN_CACHE.get(key)
        if plan is not None:
            _PLAN_CACHE.move_to_end(key)
            return plan
    desc, keepalive = build_desc()
    plan = _native.Plan(desc)
    del keepalive
    with _PLAN_LOCK:
        _PLAN_CACHE[key] = plan
        while len(_PLAN_CACHE) > _PLAN_CACHE_SIZE:
            _PLAN_CACHE.popitem(last=False)
    return plan


class Backprop3D:
    """A prepared 3D backpropagation for one sinogram shape and geometry.

    Parameters mirror ``backpropagate_3d`` / ``backpropagate_3d_tilted``;
    ``tilted_axis=None`` selects the rotation about y
    (odtbrain/_alg3d_bpp.py), any axis the tilted path
    (odtbrain/_alg3d_bppt.py).  ``input_dtype`` is "complex64" or
    "complex128" (the dtype of the device sinograms passed to
    :meth:`__call__`).  ``weights`` overrides the angle weights (None:
    computed from ``angles`` when ``weight_angles``).
    """

    def __init__(self, shape, angles, res, nm, lD=0, tilted_axis=None,
                 weight_angles=True, onlyreal=False, padding=(True, True),
                 padfac=1.75, padval="edge", intp_order=2,
                 save_memory=False, input_dtype="complex64", device=None,
                 weights=None, workspace_limit=None):
        torch = _torch()
        if device is None:
            if not torch.cuda.is_available():
                raise RuntimeError("odtbrain_gb300 needs a CUDA device; none "
                                   "is available (there is no CPU "
                                   "fallback)")
            device = torch.device("cuda", torch.cuda.current_device())
        device = torch.device(device)
        if device.type == "cuda" and device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = device
        A, lny, lnx = shape
        self.shape = (A, lny, lnx)
        self.onlyreal = bool(onlyreal)
        pad_mode, padval_c = _pad_mode(padding, padval)
        g = geom.padding_geometry(lny, lnx, padding, padfac)
        self.padding_geometry = g
        angles = np.asarray(angles)
        self.angles = angles
        self._res, self._nm, self._lD = float(res), float(nm), float(lD)
        self._support = None
        user_weights = weights
        if tilted_axis is None:
            kind = _native.ODT_GEOM_Y_AXIS

            def build_tables():
                return (geom.compute_angle_weights_1d(angles)
                        if weight_angles else None,
                        geom.rotation_y_geometry(angles, lnx, lnx), None)
            tkey = (device.index, "y", angles.dtype.str, angles.shape,
                    angles.tobytes(), lnx, bool(weight_angles))
        else:
            kind = _native.ODT_GEOM_AFFINE3D

            def build_tables():
                return geom.tilted_geometry(angles, tilted_axis,
                                            weight_angles, (lnx, lny, lnx))
            tkey = (device.index, "tilted", angles.dtype.str, angles.shape,
                    angles.tobytes(), np.asarray(tilted_axis,
                                                 dtype=np.float64).tobytes(),
                    lnx, lny, bool(weight_angles))
        with torch.cuda.device(device):
            dweights, dgeometry, taxis = _get_tables(tkey, build_tables)
        in_dtype = {"complex64": _native.ODT_INPUT_C64,
                    "complex128": _native.ODT_INPUT_C128}[str(input_dtype)
                                                         .replace("torch.",
                                                                  "")]
        self.input_dtype = (torch.complex64 if in_dtype ==
                            _native.ODT_INPUT_C64 else torch.complex128)
        if workspace_limit is None:
            workspace_limit = _WS_SAVE_MEMORY if save_memory else _WS_DEFAULT
        self._taxis = taxis
        taxis_key = None if taxis is None else tuple(float(t) for t in taxis)
        key = (self.device.index, A, lny, lnx, g["lNy"], g["lNx"],
               g["padyl"], g["padxl"], pad_mode, padval_c, int(intp_order),
               kind, self.onlyreal, in_dtype, float(res), float(nm),
               float(lD), taxis_key, int(workspace_limit))

        def build_desc():
            filt, phase = geom.filter_tables(A, g["lNx"], g["lNy"], res, nm,
                                             lD, tilted_axis=taxis)
            filt = np.ascontiguousarray(filt.view(np.float64))
            phase = np.ascontiguousarray(phase, dtype=np.float64)
            d = _native.Bpp3dDesc()
            d.num_angles = A
            d.ny, d.nx = lny, lnx
            d.pad_ny, d.pad_nx = g["lNy"], g["lNx"]
            d.pad_y_left, d.pad_x_left = g["padyl"], g["padxl"]
            d.pad_mode = pad_mode
            d.padval_re = float(np.real(padval_c))
            d.padval_im = float(np.imag(padval_c))
            d.intp_order = int(intp_order)
            d.geometry = kind
            d.onlyreal = int(self.onlyreal)
            d.input_dtype = in_dtype
            d.filter = filt.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            d.kz_phase = phase.ctypes.data_as(
                ctypes.POINTER(ctypes.c_double))
            d.workspace_limit = int(workspace_limit)
            return d, (filt, phase)

        with torch.cuda.device(self.device):
            self.plan = _get_plan(key, build_desc)
            self.weights = dweights
            if user_weights is not None:
                self.weights = torch.from_numpy(np.ascontiguousarray(
                    user_weights, dtype=np.float64)).to(self.device)
            self.geometry = dgeometry
            self.workspace = torch.empty(max(self.plan.workspace_bytes, 1),
                                         device=self.device,
                                         dtype=torch.uint8)

    @property
    def launches_per_call(self):
        return self.plan.launches_per_execute

    def volume_shape(self):
        A, lny, lnx = self.shape
        return (lnx, lny, lnx)

    def _args(self, sino, out):
        torch = _torch()
        if not (sino.is_cuda and sino.device == self.device):
            raise ValueError("sinogram must be a tensor on %s" % self.device)
        if sino.dtype != self.input_dtype or tuple(sino.shape) != self.shape:
            raise ValueError("sinogram must be %s of shape %s" %
                             (self.input_dtype, self.shape))
        if not sino.is_contiguous():
            raise ValueError("sinogram must be contiguous")
        vdtype = torch.float32 if self.onlyreal else torch.complex64
        if out is None:
            out = torch.empty(self.volume_shape(), device=self.device,
                              dtype=vdtype)
        elif (not out.is_cuda or out.device != self.device
              or out.dtype != vdtype
              or tuple(out.shape) != self.volume_shape()
              or not out.is_contiguous()):
            raise ValueError("out must be a contiguous %s tensor of shape %s "
                             "on %s" % (vdtype, self.volume_shape(),
                                        self.device))
        stream = torch.cuda.current_stream(self.device)
        args = (ctypes.c_void_p(sino.data_ptr()),
                ctypes.c_void_p(self.weights.data_ptr()
                                if self.weights is not None else 0),
                ctypes.c_void_p(self.geometry.data_ptr()),
                ctypes.c_void_p(out.data_ptr()),
                ctypes.c_void_p(self.workspace.data_ptr()),
                ctypes.c_void_p(stream.cuda_stream))
        return out, stream, args

    def __call__(self, sino, out=None, check=True):
        """Reconstruct from a device sinogram; stream-ordered on the current
        stream of the instance's device.  ``check`` waits for the stream and
        raises if a kernel recorded a failed internal check."""
        torch = _torch()
        with torch.cuda.device(self.device):
            out, stream, args = self._args(sino, out)
            self.plan.execute(*args)
            if check:
                self.plan.read_status(ctypes.c_void_p(stream.cuda_stream))
        return out

    def forward_gain(self, sino, gain=None, angle_gain=None, out=None,
                     check=True):
        """Reconstruct with gains multiplying the filter: ``gain`` a real
        (lNy, lNx) float32 map shared by all angles, ``angle_gain`` a
        complex64 (A, lNy, lNx) map per angle (None: no gain)."""
        torch = _torch()
        with torch.cuda.device(self.device):
            out, stream, args = self._args(sino, out)
            gptr = ctypes.c_void_p(self._check_gain(gain).data_ptr()
                                   if gain is not None else 0)
            aptr = ctypes.c_void_p(
                self._check_angle_gain(angle_gain).data_ptr()
                if angle_gain is not None else 0)
            self.plan.execute_gain(args[0], args[1], args[2], gptr, aptr,
                                   args[3], args[4], args[5])
            if check:
                self.plan.read_status(ctypes.c_void_p(stream.cuda_stream))
        return out

    def filter_support(self):
        """Flat positions ky*lNx + kx (int32, ascending) where the filter is
        nonzero: the only positions where a gain has an effect."""
        if self._support is None:
            g = self.padding_geometry
            filt, _ph = geom.filter_tables(self.shape[0], g["lNx"], g["lNy"],
                                           self._res, self._nm, self._lD,
                                           tilted_axis=self._taxis)
            self._support = np.flatnonzero(filt.reshape(-1) != 0).astype(
                np.int32)
        return self._support

    def gain_shape(self):
        g = self.padding_geometry
        return (g["lNy"], g["lNx"])

    def _check_gain(self, gain):
        torch = _torch()
        if (not gain.is_cuda or gain.dtype != torch.float32
                or tuple(gain.shape) != self.gain_shape()
                or not gain.is_contiguous()):
            raise ValueError("gain must be a contiguous float32 CUDA tensor "
                             "of shape %s" % (self.gain_shape(),))
        return gain

    def _check_angle_gain(self, ag):
        torch = _torch()
        shape = (self.shape[0],) + self.gain_shape()
        if (not ag.is_cuda or ag.dtype != torch.complex64
                or tuple(ag.shape) != shape or not ag.is_contiguous()):
            raise ValueError("angle_gain must be a contiguous complex64 CUDA "
                             "tensor of shape %s" % (shape,))
        return ag

    def adjoint(self, sino, vol_grad, gain=None, need_sino=True,
                need_gain=False, angle_gain=None, need_angle_gain=False):
        """Vector-Jacobian product of :meth:`forward_gain`: returns
        (sino_grad, gain_grad) -- or (sino_grad, gain_grad,
        angle_gain_grad) when ``need_angle_gain`` -- for the volume cotangent
        ``vol_grad`` (complex64, volume shape); entries not asked for are
        None."""
        torch = _torch()
        if self.onlyreal:
            raise NotImplementedError("the adjoint needs onlyreal=False")
        if (vol_grad.dtype != torch.complex64
                or tuple(vol_grad.shape) != self.volume_shape()):
            raise ValueError("vol_grad must be complex64 of the volume shape")
        vol_grad = vol_grad.contiguous()
        ws_bytes = self.plan.adjoint_workspace_bytes()
        ws = torch.empty(max(ws_bytes, 1), device=self.device,
                         dtype=torch.uint8)
        sgrad = (torch.empty(self.shape, device=self.device,
                             dtype=torch.complex64) if need_sino else None)
        ggrad = (torch.empty(self.gain_shape(), device=self.device,
                             dtype=torch.float32) if need_gain else None)
        aggrad = (torch.empty((self.shape[0],) + self.gain_shape(),
                              device=self.device, dtype=torch.complex64)
                  if need_angle_gain else None)
        stream = torch.cuda.current_stream(self.device)
        if need_gain or need_angle_gain:
            _o, _s, args = self._args(sino, vol_grad)
            sptr = args[0]
        else:
            sptr = ctypes.c_void_p(sino.data_ptr() if sino is not None
                                   else 0)
        gptr = ctypes.c_void_p(self._check_gain(gain).data_ptr()
                               if gain is not None else 0)
        aptr = ctypes.c_void_p(self._check_angle_gain(angle_gain).data_ptr()
                               if angle_gain is not None else 0)

        def ptr(t):
            return ctypes.c_void_p(t.data_ptr() if t is not None else 0)
        with torch.cuda.device(self.device):
            self.plan.adjoint(
                sptr, ptr(self.weights), ptr(self.geometry), gptr, aptr,
                ptr(vol_grad), ptr(sgrad), ptr(ggrad), ptr(aggrad), ptr(ws),
                ctypes.c_void_p(stream.cuda_stream))
            self.plan.read_status(ctypes.c_void_p(stream.cuda_stream))
        del ws
        if need_angle_gain:
            return sgrad, ggrad, aggrad
        return sgrad, ggrad

    def timed(self, sino, out=None):
        """Run once with a CUDA event pair around every kernel launch;
        returns per-stage {"ms", "launches", "bytes"}."""
        torch = _torch()
        with torch.cuda.device(self.device):
            out, stream, args = self._args(sino, out)
            t = self.plan.execute_timed(*args)
            self.plan.read_status(ctypes.c_void_p(stream.cuda_stream))
        return t

    def check(self):
        """Wait for the current stream and raise if a kernel of the plan
        recorded a failed internal check.  The status word belongs to the
        native plan, which instances of the same shape and parameters share
        (a per-process cache): a check raised here may come from another
        such instance's execution, and reading it clears it for all."""
        torch = _torch()
        with torch.cuda.device(self.device):
            stream = torch.cuda.current_stream(self.device)
            self.plan.read_status(ctypes.c_void_p(stream.cuda_stream))


def _upload(uSin, device):
    torch = _torch()
    if _is_tensor(uSin):
        t = uSin.to(device)
        if t.dtype not in (torch.complex64, torch.complex128):
            t = t.to(torch.complex128 if t.dtype == torch.float64
                     else torch.complex64)
        return t.contiguous()
    arr = np.asarray(uSin)
    if arr.dtype not in (np.complex64, np.complex128):
        arr = arr.astype(np.complex128 if arr.dtype == np.float64
                         else np.complex64)
    t = torch.from_numpy(np.ascontiguousarray(arr))
    return t.to(device, non_blocking=t.is_pinned())


def _device_for(uSin):
    torch = _torch()
    if _is_tensor(uSin) and uSin.is_cuda:
        return uSin.device
    if not torch.cuda.is_available():
        raise RuntimeError("odtbrain_gb300 needs a CUDA device; none is "
                           "available (there is no CPU fallback)")
    return torch.device("cuda", torch.cuda.current_device())


def _to_host(t):
    """Device tensor -> NumPy array through pinned host memory (torch's
    caching host allocator: the copy runs at full link speed, and the block
    is reused once the returned array is dropped)."""
    torch = _torch()
    host = torch.empty(t.shape, dtype=t.dtype, pin_memory=True)
    host.copy_(t, non_blocking=True)
    torch.cuda.current_stream(t.device).synchronize()
    return host.numpy()


def _finish(vol, uSin, dtype, onlyreal):
    torch = _torch()
    if _is_tensor(uSin):
        if onlyreal:
            return vol if dtype == np.float32 else vol.to(torch.float64)
        return vol if dtype == np.float32 else vol.to(torch.complex128)
    out = _to_host(vol)
    if onlyreal:
        return out if dtype == np.float32 else out.astype(np.float64)
    return out if dtype == np.float32 else out.astype(np.complex128)


def _apply_weights_inplace(uSin, weights):
    """copy=False: the reference multiplies the caller's array in place
    (odtbrain/_alg3d_bpp.py:272, 311-313)."""
    if _is_tensor(uSin):
        torch = _torch()
        w = torch.as_tensor(weights.reshape(-1, 1, 1), dtype=torch.float64)
        w = w.to(uSin.device).to(uSin.real.dtype if uSin.is_complex()
                                 else uSin.dtype)
        uSin.mul_(w)
    elif isinstance(uSin, np.ndarray):
        uSin *= weights.reshape(-1, 1, 1)


def _run(uSin, angles, res, nm, lD, tilted_axis, weight_angles, onlyreal,
         padding, padfac, padval, intp_order, save_memory, copy, dtype,
         count):
    torch = _torch()
    dev = _device_for(uSin)
    weights = None
    flat = np.squeeze(angles) if tilted_axis is not None else angles
    if weight_angles and len(np.shape(flat)) == 1:
        weights = geom.compute_angle_weights_1d(flat)
    with torch.cuda.device(dev):
        if weights is not None and not copy:
            # the caller's array now carries the weights; none on the GPU
            _apply_weights_inplace(uSin, weights)
            weights = None
            weight_angles = False
        t = _upload(uSin, dev)
        rec = Backprop3D(tuple(t.shape), angles, res, nm, lD=lD,
                         tilted_axis=tilted_axis,
                         weight_angles=weight_angles, onlyreal=onlyreal,
                         padding=padding, padfac=padfac, padval=padval,
                         intp_order=intp_order, save_memory=save_memory,
                         input_dtype=str(t.dtype).replace("torch.", ""),
                         device=dev, weights=weights)
        if count is not None:
            count.value += 2
        vol = rec(t)
        if count is not None:
            count.value += len(t)
    return _finish(vol, uSin, dtype, onlyreal)


def backpropagate_3d(uSin, angles, res, nm, lD=0, coords=None,
                     weight_angles=True, onlyreal=False,
                     padding=(True, True), padfac=1.75, padval="edge",
                     intp_order=2, dtype=None,
                     num_cores=ncores,
                     save_memory=False,
                     copy=True,
                     count=None, max_count=None,
                     verbose=0):
    r"""3D backpropagation about the y axis (drop-in for
    ``odtbrain.backpropagate_3d``, odtbrain/_alg3d_bpp.py:84-555).

    Parameters are those of the reference.  ``num_cores`` is validated as
    in the reference and otherwise unused; ``save_memory`` selects a smaller
    GPU workspace (more, smaller angle batches) with an identical result.

    Returns ``f`` of shape (Nx, Ny, Nx), indexed [z, y, x]: complex64 or
    complex128 per ``dtype`` (float32/float64 when ``onlyreal``).

    For ``intp_order`` 0 and 1 the reference's in-place rotation corrupts
    its result; this function computes the documented out-of-place
    rotation (what ``backpropagate_3d_tilted`` computes for the y axis).
    """
    if _is_tensor(angles):
        angles = angles.detach().cpu().numpy()
    angles = np.asarray(angles)
    A = angles.size
    shape = tuple(uSin.shape)
    dtype = _validate_common(shape, A, padding, coords, num_cores, dtype)
    _pad_mode(padding, padval)
    if max_count is not None:
        max_count.value += A + 2
    if verbose > 0:
        g = geom.padding_geometry(shape[1], shape[2], padding, padfac)
        print("......Image size (x,y): {}x{}, padded: {}x{}".format(
            shape[2], shape[1], g["lNx"], g["lNy"]))
    return _run(uSin, angles.reshape(-1), res, nm, lD, None, weight_angles,
                onlyreal, padding, padfac, padval, intp_order, save_memory,
                copy, dtype, count)


def backpropagate_3d_tilted(uSin, angles, res, nm, lD=0,
                            tilted_axis=[0, 1, 0],
                            coords=None, weight_angles=True, onlyreal=False,
                            padding=(True, True), padfac=1.75, padval="edge",
                            intp_order=2, dtype=None,
                            num_cores=ncores,
                            save_memory=False,
                            copy=True,
                            count=None, max_count=None,
                            verbose=0):
    r"""3D backpropagation with a tilted axis of rotation (drop-in for
    ``odtbrain.backpropagate_3d_tilted``, odtbrain/_alg3d_bppt.py:374-949).

    ``angles`` has shape (A,), (A, 1) or (A, 3) (points on the unit
    sphere).  Returns ``f`` of shape (Nx, Ny, Nx), indexed [z, y, x].
    """
    if _is_tensor(angles):
        angles = angles.detach().cpu().numpy()
    angles = np.asarray(angles)
    A = angles.shape[0]
    if angles.shape not in [(A,), (A, 1), (A, 3)]:
        raise ValueError("`angles` must have shape (A,) or (A,3)!")
    shape = tuple(uSin.shape)
    dtype = _validate_common(shape, A, padding, coords, num_cores, dtype)
    _pad_mode(padding, padval)
    if max_count is not None:
        max_count.value += A + 2
    if verbose > 0:
        g = geom.padding_geometry(shape[1], shape[2], padding, padfac)
        print("......Image size (x,y): {}x{}, padded: {}x{}".format(
            shape[2], shape[1], g["lNx"], g["lNy"]))
    if len(np.squeeze(angles).shape) != 1 and weight_angles:
        warnings.warn("3D angular weighting not yet supported!")
    return _run(uSin, angles, res, nm, lD, tilted_axis, weight_angles,
                onlyreal, padding, padfac, padval, intp_order, save_memory,
                copy, dtype, count)
