"""Drop-in sinogram preparation (odtbrain/_prepare_sino.py).

``sinogram_as_rytov`` (:105-182), ``sinogram_as_radon`` (:60-102) and the
helpers ``align_unwrapped`` (:7-46) and ``divmod_neg`` (:49-57), with the
phase, the unwrapping, the alignment and the Rytov composition on the GPU
(``odt_sino_prepare`` of the C ABI):

* 2D sinograms (A, N): ``numpy.unwrap`` along each detector line, in
  NumPy's operation order;
* 3D sinograms (A, Ny, Nx): per frame the reliability-sorted unwrapping
  that ``skimage.restoration.unwrap_phase(..., rng=47)`` implements
  (Herraez et al. 2002), built as the minimum spanning tree of the edge
  reliabilities.  Two things the reference leaves to its C library are
  fixed here: the large values of border pixels come from an integer hash
  of (seed, pixel) instead of ``rand()``, and equal edge weights go in edge
  index order.  The whole-turn offset of each unwrapped frame follows the
  pixel that starts the first group; ``align=True`` (the default) removes
  per-frame offsets entirely.

Arithmetic in the precision NumPy would use for ``uSin / u0``: FP32 for
complex64 / float32 data with a Python-scalar ``u0``, FP64 otherwise.
NumPy input gives NumPy output; torch tensors give CUDA tensors.  There is
no CPU fallback.
"""
import ctypes

import numpy as np

from . import _native
from ._alg3d import _device_for, _is_tensor, _to_host, _torch

SEED = 47  # the rng the reference passes to unwrap_phase


def divmod_neg(a, b):
    """Return divmod with closest result to zero (host scalar helper,
    odtbrain/_prepare_sino.py:49-57)."""
    q, r = divmod(a, b)
    sr = np.sign(r)
    if np.abs(r) > b / 2:
        q += sr
        r -= b * sr
    return q, r


def _complex_dtype(dt):
    dt = np.dtype(dt)
    if dt.kind == "c":
        return np.dtype(np.complex64) if dt.itemsize <= 8 else \
            np.dtype(np.complex128)
    if dt.kind == "f" and dt.itemsize <= 4:
        return np.dtype(np.complex64)
    return np.dtype(np.complex128)


def _np_dtype(t):
    torch = _torch()
    return {torch.float16: np.float16, torch.bfloat16: np.float32,
            torch.float32: np.float32, torch.float64: np.float64,
            torch.complex64: np.complex64, torch.complex128: np.complex128,
            }.get(t.dtype, np.float64)


def _as_device(x, dev, cdtype):
    torch = _torch()
    tdt = torch.complex64 if cdtype == np.complex64 else torch.complex128
    if _is_tensor(x):
        t = x.to(dev)
        if t.dtype == torch.bool or not (t.is_floating_point()
                                         or t.is_complex()):
            t = t.to(torch.float64)
        return t.to(tdt).contiguous()
    arr = np.ascontiguousarray(np.asarray(x).astype(cdtype, copy=False))
    return torch.from_numpy(arr).to(dev)


class SinogramPrep:
    """Prepared sinogram conversion for a fixed shape and precision on one
    CUDA device (workspace allocated once); :meth:`__call__` takes a device
    tensor.

    kind: "rytov" (complex in, complex out), "radon" (complex in, real
    out), "unwrap" or "align" (real in, real out)."""

    KINDS = {"rytov": _native.ODT_SINO_RYTOV, "radon": _native.ODT_SINO_RADON,
             "align": _native.ODT_SINO_ALIGN,
             "unwrap": _native.ODT_SINO_UNWRAP}

    def __init__(self, shape, kind="rytov", align=True, single=True, u0=1,
                 device=None):
        torch = _torch()
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        device = torch.device(device)
        if device.type == "cuda" and device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = device
        self.shape = tuple(int(v) for v in shape)
        self.kind = kind
        code = self.KINDS[kind]
        real = kind in ("align", "unwrap")
        if real:
            dcode = _native.ODT_DATA_F32 if single else _native.ODT_DATA_F64
            self.in_dtype = torch.float32 if single else torch.float64
        else:
            dcode = _native.ODT_DATA_C64 if single else _native.ODT_DATA_C128
            self.in_dtype = torch.complex64 if single else torch.complex128
        self.out_dtype = (self.in_dtype if kind in ("rytov", "align",
                                                     "unwrap")
                          else (torch.float32 if single else torch.float64))
        self.desc = _desc(self.shape, dcode, code, align)
        self._u0 = None
        if kind == "rytov":
            if _is_tensor(u0):
                self._u0 = u0.to(device=device, dtype=self.in_dtype) \
                    .expand(self.shape).contiguous()
                self.desc.u0 = self._u0.data_ptr()
            else:
                self.desc.u0_re = float(np.real(u0))
                self.desc.u0_im = float(np.imag(u0))
        L = _native.lib()
        ws_bytes = ctypes.c_uint64()
        _native.check(L.odt_sino_workspace_size(ctypes.byref(self.desc),
                                                ctypes.byref(ws_bytes)))
        self.workspace_bytes = ws_bytes.value
        n = ctypes.c_int32()
        _native.check(L.odt_sino_launch_count(ctypes.byref(self.desc),
                                              ctypes.byref(n)))
        self.launches_per_call = n.value
        with torch.cuda.device(device):
            self.workspace = torch.empty(max(ws_bytes.value, 1),
                                         dtype=torch.uint8, device=device)

    def __call__(self, sino, out=None, check=True):
        torch = _torch()
        if (not sino.is_cuda or sino.device != self.device
                or sino.dtype != self.in_dtype
                or tuple(sino.shape) != self.shape):
            raise ValueError("input must be %s of shape %s on %s"
                             % (self.in_dtype, self.shape, self.device))
        sino = sino.contiguous()
        if out is None:
            out = torch.empty(self.shape, dtype=self.out_dtype,
                              device=self.device)
        elif (out.dtype != self.out_dtype or tuple(out.shape) != self.shape
              or out.device != self.device or not out.is_contiguous()):
            raise ValueError("out must be a contiguous %s tensor of shape %s"
                             % (self.out_dtype, self.shape))
        L = _native.lib()
        stream = torch.cuda.current_stream(self.device)
        sp = ctypes.c_void_p(stream.cuda_stream)
        wp = ctypes.c_void_p(self.workspace.data_ptr())
        _native.check(L.odt_sino_prepare(
            ctypes.byref(self.desc), ctypes.c_void_p(sino.data_ptr()),
            ctypes.c_void_p(out.data_ptr()), wp, self.workspace_bytes, sp))
        if check:
            _native.check(L.odt_sino_read_status(wp, sp))
        return out


def _desc(shape, dtype_code, kind, align):
    d = _native.SinoDesc()
    d.num_angles = shape[0]
    d.ny = shape[1] if len(shape) == 3 else 0
    d.nx = shape[-1]
    d.dtype = dtype_code
    d.kind = kind
    d.align = int(bool(align))
    d.seed = SEED
    return d


def _run(kind, uSin, u0, align):
    torch = _torch()
    is_t = _is_tensor(uSin)
    in_dt = _np_dtype(uSin) if is_t else np.asarray(uSin).dtype
    shape = tuple(uSin.shape)
    if len(shape) < 2:
        raise ValueError("Image must be 1, 2, or 3 dimensional")
    if len(shape) > 3:
        raise NotImplementedError("sinograms of 3D volumes (4D input) are not "
                                  "supported")
    rytov = kind == "rytov"
    if rytov:
        if _is_tensor(u0) or isinstance(u0, np.ndarray):
            u0_dt = _np_dtype(u0) if _is_tensor(u0) else u0.dtype
            res_dt = np.result_type(in_dt, u0_dt)
        else:
            res_dt = np.result_type(in_dt, u0)
    else:
        res_dt = in_dt
    cdt = _complex_dtype(res_dt)
    dev = _device_for(uSin)
    with torch.cuda.device(dev):
        sino = _as_device(uSin, dev, cdt)
        if rytov and (_is_tensor(u0) or isinstance(u0, np.ndarray)):
            u0 = _as_device(u0, dev, cdt)
            try:
                bshape = tuple(torch.broadcast_shapes(u0.shape, sino.shape))
            except RuntimeError:
                bshape = None
            if bshape != shape:
                # NumPy raises ValueError for operands that do not broadcast
                raise ValueError("u0 of shape %s does not broadcast to the "
                                 "sinogram's %s" % (tuple(u0.shape), shape))
        prep = SinogramPrep(shape, kind, align, single=cdt == np.complex64,
                            u0=u0 if rytov else 1, device=dev)
        out = prep(sino)
    if is_t:
        return out
    return _to_host(out)


def _real_inplace(kind, phase, align):
    """Run a real-phase mode ("align" / "unwrap") on ``phase`` (NumPy array
    or CUDA tensor of float32 / float64) in place on a device copy; returns
    the device result and whether the input was a tensor."""
    torch = _torch()
    is_t = _is_tensor(phase)
    if is_t:
        if phase.dtype not in (torch.float32, torch.float64):
            raise ValueError("phase must be float32 or float64")
        single = phase.dtype == torch.float32
    else:
        dt = np.asarray(phase).dtype
        if dt not in (np.float32, np.float64):
            raise ValueError("phase must be float32 or float64")
        single = dt == np.float32
    shape = tuple(phase.shape)
    if len(shape) not in (2, 3):
        raise ValueError("phase must have 2 or 3 dimensions")
    dev = _device_for(phase)
    with torch.cuda.device(dev):
        t = (phase.to(dev) if is_t else torch.from_numpy(
            np.ascontiguousarray(phase)).to(dev)).contiguous()
        SinogramPrep(shape, kind, align, single=single, device=dev)(t, out=t)
    return t, is_t


def sinogram_as_rytov(uSin, u0=1, align=True):
    r"""Convert the complex wave field sinogram to the Rytov phase (drop-in
    for ``odtbrain.sinogram_as_rytov``, odtbrain/_prepare_sino.py:105-182).

    Returns ``u0 * (log|uSin/u0| + 1j * unwrap(angle(uSin/u0)))``, aligned
    with :func:`align_unwrapped` when ``align``."""
    return _run("rytov", uSin, u0, align)


def sinogram_as_radon(uSin, align=True):
    r"""Unwrapped phase of a complex wave field sinogram (drop-in for
    ``odtbrain.sinogram_as_radon``, odtbrain/_prepare_sino.py:60-102)."""
    return _run("radon", uSin, None, align)


def align_unwrapped(sino):
    """Align an unwrapped phase sinogram (A, N) or (A, Ny, Nx) to zero phase,
    in place (odtbrain/_prepare_sino.py:7-46): per-angle whole-turn steps by
    majority vote of five border samples unwrapped along the angle axis,
    then the whole turns of the global minimum.  Works on a NumPy array or a
    CUDA tensor of float32 / float64; the computation runs on the GPU."""
    t, is_t = _real_inplace("align", sino, True)
    if is_t:
        if t.data_ptr() != sino.data_ptr():
            sino.copy_(t)
    else:
        sino[...] = t.cpu().numpy()


def unwrap_frames(phase):
    """Reliability-sorted 2D phase unwrapping of one frame (Ny, Nx) or of
    every frame of a stack (A, Ny, Nx): the algorithm of
    ``skimage.restoration.unwrap_phase`` for 2D images (Herraez et al.
    2002), as ``sinogram_as_rytov`` applies it with ``rng=47``
    (odtbrain/_prepare_sino.py:171-172).  float32 / float64, NumPy or CUDA
    tensor in, same out (a new array)."""
    one = len(tuple(phase.shape)) == 2
    src = phase[None] if one else phase
    t, is_t = _real_inplace("unwrap", src.clone()
                            if _is_tensor(src) else src, False)
    if one:
        t = t[0]
    if is_t:
        return t
    return t.cpu().numpy()
