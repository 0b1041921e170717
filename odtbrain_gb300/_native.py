"""ctypes binding of the C ABI in ``include/odtbrain_gb300.h``.

The shared library is built in-tree by ``odtbrain_gb300.build`` and loaded
from ``odtbrain_gb300/_lib``.  There is no CPU fallback: if the library is
missing, :func:`lib` raises.
"""
import ctypes
import os
import threading

from . import build as _build

ODT_OK = 0
ODT_ERR_INVALID_ARGUMENT = 1
ODT_ERR_UNSUPPORTED = 2
ODT_ERR_CUDA = 3
ODT_ERR_OUT_OF_MEMORY = 4
ODT_ERR_DEVICE_CHECK = 5

ODT_PAD_NONE, ODT_PAD_EDGE, ODT_PAD_RAMP = 0, 1, 2
ODT_GEOM_Y_AXIS, ODT_GEOM_AFFINE3D = 0, 1
ODT_INPUT_C64, ODT_INPUT_C128 = 0, 1
ODT_DATA_F32, ODT_DATA_F64, ODT_DATA_C64, ODT_DATA_C128 = 0, 1, 2, 3
ODT_SINO_RYTOV, ODT_SINO_RADON, ODT_SINO_ALIGN, ODT_SINO_UNWRAP = 0, 1, 2, 3
ODT_APPLE_NN, ODT_APPLE_SH, ODT_APPLE_NONE = 0, 1, 2
# size of the static scratch of odt_bpp3d_execute_noalloc
NOALLOC_SCRATCH_BYTES = 64 << 20

# every symbol include/odtbrain_gb300.h declares
EXPORTED_SYMBOLS = (
    "odt_bpp3d_plan_create",
    "odt_bpp3d_workspace_size",
    "odt_bpp3d_angle_batch",
    "odt_bpp3d_execute",
    "odt_bpp3d_execute_timed",
    "odt_bpp3d_launch_count",
    "odt_bpp3d_execute_noalloc",
    "odt_bpp3d_execute_gain",
    "odt_bpp3d_adjoint_workspace_size",
    "odt_bpp3d_adjoint",
    "odt_bpp3d_read_status",
    "odt_bpp3d_plan_destroy",
    "odt_mlp_gain_forward",
    "odt_mlp_store_size",
    "odt_mlp_gain_backward",
    "odt_mlp_read_status",
    "odt_mlp_select_kernels",
    "odt_odt_to_ri",
    "odt_opt_to_ri",
    "odt_sino_workspace_size",
    "odt_sino_prepare",
    "odt_sino_launch_count",
    "odt_sino_read_status",
    "odt_apple_workspace_size",
    "odt_apple_correct",
    "odt_apple_flags",
    "odt_apple_flags_workspace_size",
    "odt_apple_constrain_workspace_size",
    "odt_apple_constrain",
    "odt_apple_envelope_workspace_size",
    "odt_apple_envelope",
    "odt_debug_inject_status",
    "odt_debug_set_table_alloc_limit",
    "odt_status_string",
    "odt_last_error",
)


class OdtError(RuntimeError):
    """A non-OK status returned by the native library."""

    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


class Bpp3dDesc(ctypes.Structure):
    _fields_ = [
        ("num_angles", ctypes.c_int32),
        ("ny", ctypes.c_int32),
        ("nx", ctypes.c_int32),
        ("pad_ny", ctypes.c_int32),
        ("pad_nx", ctypes.c_int32),
        ("pad_y_left", ctypes.c_int32),
        ("pad_x_left", ctypes.c_int32),
        ("pad_mode", ctypes.c_int32),
        ("padval_re", ctypes.c_double),
        ("padval_im", ctypes.c_double),
        ("intp_order", ctypes.c_int32),
        ("geometry", ctypes.c_int32),
        ("onlyreal", ctypes.c_int32),
        ("input_dtype", ctypes.c_int32),
        ("filter", ctypes.POINTER(ctypes.c_double)),
        ("kz_phase", ctypes.POINTER(ctypes.c_double)),
        ("workspace_limit", ctypes.c_uint64),
        ("z_shift", ctypes.c_double),
    ]


class MlpParams(ctypes.Structure):
    """odt_mlp_params: device pointers of the BF16 weights (and transposes)
    and FP32 biases of the learned-gain MLP."""
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("w1", "w2", "w3", "w4", "w2t", "w3t", "w4t",
                 "b1", "b2", "b3", "b4")]


class MlpGrads(ctypes.Structure):
    """odt_mlp_grads: FP32 device gradient buffers (accumulated)."""
    _fields_ = [(n, ctypes.c_void_p) for n in
                ("w1", "w2", "w3", "w4", "b1", "b2", "b3", "b4")]


STAGE_NAMES = ("rows_forward", "columns_propagate", "rows_inverse",
               "rotate")


class SinoDesc(ctypes.Structure):
    """odt_sino_desc of include/odtbrain_gb300.h."""
    _fields_ = [
        ("num_angles", ctypes.c_int64),
        ("ny", ctypes.c_int32),
        ("nx", ctypes.c_int32),
        ("dtype", ctypes.c_int32),
        ("kind", ctypes.c_int32),
        ("align", ctypes.c_int32),
        ("seed", ctypes.c_uint32),
        ("u0", ctypes.c_void_p),
        ("u0_re", ctypes.c_double),
        ("u0_im", ctypes.c_double),
    ]


class AppleDesc(ctypes.Structure):
    """odt_apple_desc of include/odtbrain_gb300.h."""
    _fields_ = [
        ("n0", ctypes.c_int32),
        ("n1", ctypes.c_int32),
        ("n2", ctypes.c_int32),
        ("res", ctypes.c_double),
        ("nm", ctypes.c_double),
        ("method", ctypes.c_int32),
        ("enforce_envelope", ctypes.c_double),
        ("max_iter", ctypes.c_int32),
        ("min_diff", ctypes.c_double),
        ("use_bg_shell", ctypes.c_int32),
        ("bg_shell_width", ctypes.c_double),
        ("gauss_radius", ctypes.c_int32),
        ("gauss_weights", ctypes.POINTER(ctypes.c_double)),
    ]


class StageTiming(ctypes.Structure):
    _fields_ = [
        ("ms", ctypes.c_double * 4),
        ("launches", ctypes.c_int64 * 4),
        ("bytes", ctypes.c_double * 4),
    ]

    def as_dict(self):
        return {name: {"ms": self.ms[i], "launches": int(self.launches[i]),
                       "bytes": self.bytes[i]}
                for i, name in enumerate(STAGE_NAMES)}


_LIB = None
_LOCK = threading.Lock()


def library_path():
    return _build.LIB


def lib():
    """Load (once) and return the native library; raises if it is absent."""
    global _LIB
    if _LIB is not None:
        return _LIB
    with _LOCK:
        if _LIB is not None:
            return _LIB
        path = _build.LIB
        if not os.path.exists(path):
            raise RuntimeError(
                "odtbrain_gb300 CUDA library not built (%s missing); run "
                "`python -m odtbrain_gb300.build` or "
                "`python -c 'import __graft_entry__ as g; g.build()'`" % path)
        L = ctypes.CDLL(path)
        vp = ctypes.c_void_p
        L.odt_bpp3d_plan_create.argtypes = [ctypes.POINTER(Bpp3dDesc),
                                            ctypes.POINTER(vp)]
        L.odt_bpp3d_workspace_size.argtypes = [
            vp, ctypes.POINTER(ctypes.c_uint64)]
        L.odt_bpp3d_angle_batch.argtypes = [vp,
                                            ctypes.POINTER(ctypes.c_int32)]
        L.odt_bpp3d_execute.argtypes = [vp, vp, vp, vp, vp, vp, vp]
        L.odt_bpp3d_execute_timed.argtypes = [vp, vp, vp, vp, vp, vp, vp,
                                              ctypes.POINTER(StageTiming)]
        L.odt_bpp3d_launch_count.argtypes = [vp,
                                             ctypes.POINTER(ctypes.c_int64)]
        L.odt_bpp3d_execute_noalloc.argtypes = [vp, vp, vp, vp, vp, vp]
        L.odt_bpp3d_execute_gain.argtypes = [vp, vp, vp, vp, vp, vp, vp, vp,
                                             vp]
        L.odt_bpp3d_adjoint_workspace_size.argtypes = [
            vp, ctypes.POINTER(ctypes.c_uint64)]
        L.odt_bpp3d_adjoint.argtypes = [vp] * 12
        L.odt_bpp3d_read_status.argtypes = [vp, vp]
        L.odt_bpp3d_plan_destroy.argtypes = [vp]
        L.odt_debug_inject_status.argtypes = [vp, ctypes.c_int32, vp]
        L.odt_debug_set_table_alloc_limit.argtypes = [ctypes.c_uint64]
        for name in ("odt_odt_to_ri", "odt_opt_to_ri"):
            getattr(L, name).argtypes = [vp, vp, ctypes.c_int64,
                                         ctypes.c_int32, ctypes.c_double,
                                         ctypes.c_double, vp]
        sd = ctypes.POINTER(SinoDesc)
        L.odt_sino_workspace_size.argtypes = [
            sd, ctypes.POINTER(ctypes.c_uint64)]
        L.odt_sino_prepare.argtypes = [sd, vp, vp, vp, ctypes.c_uint64, vp]
        L.odt_sino_launch_count.argtypes = [sd,
                                            ctypes.POINTER(ctypes.c_int32)]
        L.odt_sino_read_status.argtypes = [vp, vp]
        ad = ctypes.POINTER(AppleDesc)
        L.odt_apple_workspace_size.argtypes = [
            ad, ctypes.POINTER(ctypes.c_uint64)]
        L.odt_apple_correct.argtypes = [ad, vp, vp, vp, vp, ctypes.c_uint64,
                                        ctypes.POINTER(ctypes.c_int32), vp]
        L.odt_apple_flags.argtypes = [ad, vp, vp, vp, vp]
        L.odt_apple_flags_workspace_size.argtypes = [
            ad, ctypes.POINTER(ctypes.c_uint64)]
        i32 = ctypes.c_int32
        L.odt_apple_constrain_workspace_size.argtypes = [
            ad, ctypes.POINTER(ctypes.c_uint64)]
        L.odt_apple_constrain.argtypes = [ad, i32, i32, vp, vp, vp, vp,
                                          ctypes.c_uint64, vp]
        L.odt_apple_envelope_workspace_size.argtypes = [
            ad, ctypes.POINTER(ctypes.c_uint64)]
        L.odt_apple_envelope.argtypes = [ad, i32, vp, vp, vp, vp,
                                         ctypes.c_uint64, vp]
        L.odt_mlp_gain_forward.argtypes = [ctypes.POINTER(MlpParams), i32,
                                           i32, i32, vp, vp, i32, vp, vp]
        L.odt_mlp_read_status.argtypes = [vp]
        L.odt_mlp_select_kernels.argtypes = [i32]
        L.odt_mlp_store_size.argtypes = [i32, i32,
                                         ctypes.POINTER(ctypes.c_uint64)]
        L.odt_mlp_gain_backward.argtypes = [
            ctypes.POINTER(MlpParams), i32, i32, i32, vp, vp, i32, vp, vp,
            ctypes.POINTER(MlpGrads), vp]
        for name in ("odt_bpp3d_plan_create", "odt_bpp3d_workspace_size",
                     "odt_bpp3d_angle_batch", "odt_bpp3d_execute",
                     "odt_bpp3d_execute_timed", "odt_bpp3d_launch_count",
                     "odt_bpp3d_execute_noalloc", "odt_bpp3d_execute_gain",
                     "odt_bpp3d_adjoint_workspace_size", "odt_bpp3d_adjoint",
                     "odt_bpp3d_read_status", "odt_bpp3d_plan_destroy",
                     "odt_mlp_gain_forward", "odt_mlp_store_size",
                     "odt_mlp_gain_backward", "odt_mlp_read_status",
                     "odt_mlp_select_kernels",
                     "odt_odt_to_ri",
                     "odt_opt_to_ri", "odt_sino_workspace_size",
                     "odt_sino_prepare", "odt_sino_launch_count",
                     "odt_sino_read_status", "odt_apple_workspace_size",
                     "odt_apple_correct", "odt_apple_flags",
                     "odt_apple_flags_workspace_size",
                     "odt_apple_constrain_workspace_size",
                     "odt_apple_constrain",
                     "odt_apple_envelope_workspace_size",
                     "odt_apple_envelope",
                     "odt_debug_inject_status",
                     "odt_debug_set_table_alloc_limit"):
            getattr(L, name).restype = ctypes.c_int
        L.odt_status_string.argtypes = [ctypes.c_int]
        L.odt_status_string.restype = ctypes.c_char_p
        L.odt_last_error.argtypes = []
        L.odt_last_error.restype = ctypes.c_char_p
        _LIB = L
        return L


def set_table_alloc_limit(nbytes):
    """Test hook: make plan creation fail with MemoryError when its device
    tables exceed `nbytes` (0 removes the limit)."""
    check(lib().odt_debug_set_table_alloc_limit(int(nbytes)))


def check(status):
    """Raise the Python exception the reference would raise for a status."""
    if status == ODT_OK:
        return
    L = lib()
    detail = L.odt_last_error().decode(errors="replace")
    text = "%s: %s" % (L.odt_status_string(status).decode(), detail)
    if status == ODT_ERR_INVALID_ARGUMENT:
        raise ValueError(text)
    if status == ODT_ERR_UNSUPPORTED:
        raise NotImplementedError(text)
    if status == ODT_ERR_OUT_OF_MEMORY:
        raise MemoryError(text)
    raise OdtError(status, text)


class Plan:
    """Owns an ``odt_bpp3d_plan``.  A plan's executions fork onto the plan's
    own second stream, so enqueueing them is serialised per plan (the C ABI
    forbids concurrent execution of one plan from several host threads)."""

    def __init__(self, desc):
        self._lock = threading.Lock()
        L = lib()
        handle = ctypes.c_void_p()
        check(L.odt_bpp3d_plan_create(ctypes.byref(desc),
                                      ctypes.byref(handle)))
        self._h = handle
        ws = ctypes.c_uint64()
        check(L.odt_bpp3d_workspace_size(self._h, ctypes.byref(ws)))
        self.workspace_bytes = int(ws.value)
        b = ctypes.c_int32()
        check(L.odt_bpp3d_angle_batch(self._h, ctypes.byref(b)))
        self.angle_batch = int(b.value)
        n = ctypes.c_int64()
        check(L.odt_bpp3d_launch_count(self._h, ctypes.byref(n)))
        self.launches_per_execute = int(n.value)

    def execute(self, sino_ptr, weights_ptr, geometry_ptr, volume_ptr,
                workspace_ptr, stream_handle):
        with self._lock:
            check(lib().odt_bpp3d_execute(self._h, sino_ptr, weights_ptr,
                                          geometry_ptr, volume_ptr,
                                          workspace_ptr, stream_handle))

    def execute_timed(self, sino_ptr, weights_ptr, geometry_ptr, volume_ptr,
                      workspace_ptr, stream_handle):
        t = StageTiming()
        with self._lock:
            check(lib().odt_bpp3d_execute_timed(
                self._h, sino_ptr, weights_ptr, geometry_ptr, volume_ptr,
                workspace_ptr, stream_handle, ctypes.byref(t)))
        return t.as_dict()

    def execute_gain(self, sino_ptr, weights_ptr, geometry_ptr, gain_ptr,
                     again_ptr, volume_ptr, workspace_ptr, stream_handle):
        with self._lock:
            check(lib().odt_bpp3d_execute_gain(
                self._h, sino_ptr, weights_ptr, geometry_ptr, gain_ptr,
                again_ptr, volume_ptr, workspace_ptr, stream_handle))

    def adjoint_workspace_bytes(self):
        ws = ctypes.c_uint64()
        check(lib().odt_bpp3d_adjoint_workspace_size(self._h,
                                                     ctypes.byref(ws)))
        return int(ws.value)

    def adjoint(self, sino_ptr, weights_ptr, geometry_ptr, gain_ptr,
                again_ptr, vgrad_ptr, sgrad_ptr, ggrad_ptr, aggrad_ptr,
                workspace_ptr, stream_handle):
        with self._lock:
            check(lib().odt_bpp3d_adjoint(self._h, sino_ptr, weights_ptr,
                                          geometry_ptr, gain_ptr, again_ptr,
                                          vgrad_ptr, sgrad_ptr, ggrad_ptr,
                                          aggrad_ptr, workspace_ptr,
                                          stream_handle))

    def read_status(self, stream_handle):
        check(lib().odt_bpp3d_read_status(self._h, stream_handle))

    def inject_status(self, bits, stream_handle):
        """Test hook: set the plan's device status word to `bits`, as a
        kernel whose own check tripped would (odt_debug_inject_status)."""
        check(lib().odt_debug_inject_status(self._h, int(bits),
                                            stream_handle))

    def __del__(self):
        h = getattr(self, "_h", None)
        if h is not None and h.value and _LIB is not None:
            _LIB.odt_bpp3d_plan_destroy(h)
            self._h = None
