"""Drop-in ``backpropagate_2d`` (odtbrain/_alg2d_bpp.py:8-326).

The 2D algorithm is one y plane of the 3D y-axis pipeline: per angle the
padded line is Fourier transformed along x and filtered, every output row
``yv`` gets the propagator ``exp(i km (M-1) yv)`` and an inverse transform,
the result is cropped to an (ln, ln) image, rotated by ``-phi`` with
``scipy.ndimage.rotate``'s default cubic spline (prefilter included) and
summed.  So the GPU runs it as a y-axis plan with ny = 1: the host builds the
2D padding (next power of two of 2.1*ln, at least 64), the 2D filter (the
reference's normalised inverse FFT folded in as 1/lN) and the rotation
geometry in the reference's FP64 operation order, and the rows sit at
``yv = k - ln/2 + 0.5`` (``z_shift`` 0.5).

Same signature, defaults, validation (``assert`` statements, like the
reference), progress counters and output as the reference: an (ln, ln)
complex128 array (float64 when ``onlyreal``); torch tensors in give CUDA
tensors out.  The GPU arithmetic is FP32 with compensated sums.
"""
import ctypes

import numpy as np

from . import _geometry as geom
from . import _native
from ._alg3d import (_WS_DEFAULT, _device_for, _get_plan, _get_tables,
                     _is_tensor, _torch)


class Backprop2D:
    """Prepared 2D backpropagation for a fixed geometry on one CUDA device;
    :meth:`__call__` takes a device sinogram (A, ln)."""

    def __init__(self, shape, angles, res, nm, lD=0, weight_angles=True,
                 onlyreal=False, padding=True, padval=0,
                 input_dtype="complex64", device=None):
        torch = _torch()
        if device is None:
            device = torch.device("cuda", torch.cuda.current_device())
        device = torch.device(device)
        if device.type == "cuda" and device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = device
        A, ln = shape
        self.shape = (A, ln)
        self.onlyreal = bool(onlyreal)
        angles = np.asarray(angles).reshape(-1)
        g = geom.padding_geometry_2d(ln, padding)
        self.padding_geometry = g
        if not padding or g["lN"] == ln:
            pad_mode, padval_c = _native.ODT_PAD_NONE, 0j
        elif padval is None:
            pad_mode, padval_c = _native.ODT_PAD_EDGE, 0j
        else:
            pad_mode, padval_c = _native.ODT_PAD_RAMP, complex(padval)
        in_dtype = {"complex64": _native.ODT_INPUT_C64,
                    "complex128": _native.ODT_INPUT_C128}[
                        str(input_dtype).replace("torch.", "")]
        self.input_dtype = (torch.complex64 if in_dtype ==
                            _native.ODT_INPUT_C64 else torch.complex128)

        def build_tables():
            return (geom.compute_angle_weights_1d(angles) if weight_angles
                    else None, geom.rotation_2d_geometry(angles, ln), None)
        tkey = (device.index, "2d", angles.dtype.str, angles.shape,
                angles.tobytes(), ln, bool(weight_angles))
        key = ("2d", device.index, A, ln, g["lN"], g["padl"], pad_mode,
               padval_c, self.onlyreal, in_dtype, float(res), float(nm),
               float(lD))

        def build_desc():
            filt, phase = geom.filter_tables_2d(A, g["lN"], res, nm, lD)
            filt = np.ascontiguousarray(filt.view(np.float64))
            d = _native.Bpp3dDesc()
            d.num_angles = A
            d.ny, d.nx = 1, ln
            d.pad_ny, d.pad_nx = 1, g["lN"]
            d.pad_y_left, d.pad_x_left = 0, g["padl"]
            d.pad_mode = pad_mode
            d.padval_re = float(np.real(padval_c))
            d.padval_im = float(np.imag(padval_c))
            d.intp_order = 3  # scipy.ndimage.rotate's default order
            d.geometry = _native.ODT_GEOM_Y_AXIS
            d.onlyreal = int(self.onlyreal)
            d.input_dtype = in_dtype
            d.filter = filt.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
            d.kz_phase = phase.ctypes.data_as(
                ctypes.POINTER(ctypes.c_double))
            d.workspace_limit = _WS_DEFAULT
            d.z_shift = 0.5
            return d, (filt, phase)

        with torch.cuda.device(device):
            self.plan = _get_plan(key, build_desc)
            self.weights, self.geometry, _ = _get_tables(tkey, build_tables)
            self.workspace = torch.empty(max(self.plan.workspace_bytes, 1),
                                         device=device, dtype=torch.uint8)

    def __call__(self, sino, out=None, check=True):
        """Reconstruct from a device sinogram (A, ln); returns the (ln, ln)
        image (complex64, or float32 when ``onlyreal``)."""
        torch = _torch()
        A, ln = self.shape
        if (not sino.is_cuda or sino.device != self.device
                or sino.dtype != self.input_dtype
                or tuple(sino.shape) != self.shape):
            raise ValueError("sinogram must be %s of shape %s on %s"
                             % (self.input_dtype, self.shape, self.device))
        sino = sino.contiguous()
        vdtype = torch.float32 if self.onlyreal else torch.complex64
        if out is None:
            out = torch.empty((ln, ln), device=self.device, dtype=vdtype)
        elif (out.dtype != vdtype or tuple(out.shape) != (ln, ln)
              or out.device != self.device or not out.is_contiguous()):
            raise ValueError("out must be a contiguous %s tensor of shape "
                             "%s" % (vdtype, (ln, ln)))
        stream = torch.cuda.current_stream(self.device)
        self.plan.execute(
            ctypes.c_void_p(sino.data_ptr()),
            ctypes.c_void_p(self.weights.data_ptr()
                            if self.weights is not None else 0),
            ctypes.c_void_p(self.geometry.data_ptr()),
            ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(self.workspace.data_ptr()),
            ctypes.c_void_p(stream.cuda_stream))
        if check:
            self.plan.read_status(ctypes.c_void_p(stream.cuda_stream))
        return out

    @property
    def launches_per_call(self):
        return self.plan.launches_per_execute

    def timed(self, sino, out=None):
        """Run once with a CUDA event pair around every kernel launch;
        returns per-stage {"ms", "launches", "bytes"}."""
        torch = _torch()
        A, ln = self.shape
        vdtype = torch.float32 if self.onlyreal else torch.complex64
        if out is None:
            out = torch.empty((ln, ln), device=self.device, dtype=vdtype)
        self(sino, out=out, check=False)  # argument checks, warm tables
        stream = torch.cuda.current_stream(self.device)
        t = self.plan.execute_timed(
            ctypes.c_void_p(sino.data_ptr()),
            ctypes.c_void_p(self.weights.data_ptr()
                            if self.weights is not None else 0),
            ctypes.c_void_p(self.geometry.data_ptr()),
            ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(self.workspace.data_ptr()),
            ctypes.c_void_p(stream.cuda_stream))
        self.plan.read_status(ctypes.c_void_p(stream.cuda_stream))
        return t


def backpropagate_2d(uSin, angles, res, nm, lD=0, coords=None,
                     weight_angles=True,
                     onlyreal=False, padding=True, padval=0,
                     count=None, max_count=None, verbose=0):
    r"""2D backpropagation with the Fourier diffraction theorem (drop-in for
    ``odtbrain.backpropagate_2d``, odtbrain/_alg2d_bpp.py:8-326).

    Parameters are those of the reference; ``padval=None`` pads with the
    edge values.  Returns ``f`` of shape (N, N): complex128, or float64
    when ``onlyreal`` (CUDA tensors of those dtypes for tensor input).
    """
    if _is_tensor(angles):
        angles = angles.detach().cpu().numpy()
    angles = np.asarray(angles)
    A = angles.shape[0]
    if max_count is not None:
        max_count.value += A + 2
    assert len(uSin.shape) == 2, "Input data `uB` must have shape (A,N)!"
    assert len(uSin) == A, "`len(angles)` must be  equal to `len(uSin)`!"
    if coords is not None:
        # the reference builds this message with a stray unary "+" on a
        # string (odtbrain/_alg2d_bpp.py:136-137), which raises TypeError
        raise TypeError("bad operand type for unary +: 'str' (output "
                        "coordinates cannot yet be set for the 2D "
                        "backpropagation algorithm)")
    torch = _torch()
    dev = _device_for(uSin)
    ln = uSin.shape[1]
    if verbose > 0:
        print("......Padding with edge values." if padval is None
              else "......Verifying padding value: {}".format(padval))
    with torch.cuda.device(dev):
        if _is_tensor(uSin):
            t = uSin.to(dev)
            if not t.is_complex():
                t = t.to(torch.complex128 if t.dtype == torch.float64
                         else torch.complex64)
        else:
            arr = np.asarray(uSin)
            if arr.dtype not in (np.complex64, np.complex128):
                arr = arr.astype(np.complex128)
            t = torch.from_numpy(np.ascontiguousarray(arr)).to(dev)
        t = t.contiguous()
        rec = Backprop2D((A, ln), angles, res, nm, lD=lD,
                         weight_angles=weight_angles, onlyreal=onlyreal,
                         padding=padding, padval=padval,
                         input_dtype=str(t.dtype).replace("torch.", ""),
                         device=dev)
        if count is not None:
            count.value += 2
        img = rec(t)
        if count is not None:
            count.value += A
    out_dtype = torch.float64 if onlyreal else torch.complex128
    if _is_tensor(uSin):
        return img.to(out_dtype)
    return img.cpu().numpy().astype(np.float64 if onlyreal
                                    else np.complex128)
