"""Drop-in ``odt_to_ri`` and ``opt_to_ri`` (odtbrain/_translate_ri.py).

Elementwise on the GPU (``odt_odt_to_ri`` / ``odt_opt_to_ri`` of the C ABI):

* ``odt_to_ri``: n = nm * sqrt(f / km^2 + 1), km = 2 pi nm / res, the root
  with non-negative real part (complex data; NaN below -1 for real data, as
  NumPy gives);
* ``opt_to_ri``: n = nm + f / (2 pi) * res.

NumPy input gives NumPy output of the reference's dtype (integers and bools
become float64, float32/complex64 stay single precision); torch tensors give
CUDA tensors.  There is no CPU fallback.
"""
import ctypes

import numpy as np

from . import _native
from ._alg3d import _device_for, _is_tensor, _to_host, _torch

_CODES = {"float32": _native.ODT_DATA_F32, "float64": _native.ODT_DATA_F64,
          "complex64": _native.ODT_DATA_C64,
          "complex128": _native.ODT_DATA_C128}


def _apply(fn_name, f, res, nm):
    torch = _torch()
    dev = _device_for(f)
    if _is_tensor(f):
        t = f.to(dev)
        if not (t.is_floating_point() or t.is_complex()):
            t = t.to(torch.float64)
        elif t.dtype in (torch.float16, torch.bfloat16):
            t = t.to(torch.float32)
        host = None
    else:
        host = np.asarray(f)
        if host.dtype.kind in "biu":
            host = host.astype(np.float64)
        elif host.dtype == np.float16:
            host = host.astype(np.float32)
        elif host.dtype.kind not in "fc":
            raise TypeError("unsupported data type %s" % host.dtype)
        t = torch.from_numpy(np.ascontiguousarray(host)).to(dev)
    t = t.contiguous()
    out = torch.empty_like(t)
    code = _CODES[str(t.dtype).replace("torch.", "")]
    with torch.cuda.device(dev):
        stream = torch.cuda.current_stream(dev)
        _native.check(getattr(_native.lib(), fn_name)(
            ctypes.c_void_p(t.data_ptr()), ctypes.c_void_p(out.data_ptr()),
            t.numel(), code, float(res), float(nm),
            ctypes.c_void_p(stream.cuda_stream)))
    if host is not None:
        return _to_host(out)
    return out


def odt_to_ri(f, res, nm):
    r"""Convert the ODT object function to refractive index (drop-in for
    ``odtbrain.odt_to_ri``, odtbrain/_translate_ri.py:5-57)."""
    return _apply("odt_odt_to_ri", f, res, nm)


def opt_to_ri(f, res, nm):
    r"""Convert the OPT object function to refractive index (drop-in for
    ``odtbrain.opt_to_ri``, odtbrain/_translate_ri.py:60-93)."""
    return _apply("odt_opt_to_ri", f, res, nm)
