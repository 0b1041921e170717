"""The allocation-free execution entry point (``odt_bpp3d_execute_noalloc``).

Callers that cannot allocate device memory at reconstruction time (inside
a captured stream, in a latency-critical loop, or under an application
allocator that owns all device memory) run a plan with the library's
static 64 MiB device scratch instead of a workspace.  This file checks,
through the C ABI, that two calls in a row give what the workspace-based
``odt_bpp3d_execute`` gives, and that a plan needing more scratch than the
static array holds is refused with a clear error.  It is collected last so
that a stop-at-first-failure run has already run every other test.
"""
import ctypes

import numpy as np
import pytest

from sino_gen import ellipsoid_phantom_sinogram

pytestmark = pytest.mark.gpu

REL_L2 = 1e-5
MAX_REL = 1e-5


def _close(got, ref):
    got = got.cpu().numpy()
    ref = ref.cpu().numpy()
    rel = np.linalg.norm(got - ref) / np.linalg.norm(ref)
    mx = np.abs(got - ref).max() / np.abs(ref).max()
    return rel <= REL_L2 and mx <= MAX_REL, rel, mx


def test_noalloc_matches_workspace_execute(cuda_ready):
    import torch
    from odtbrain_gb300 import _native
    from odtbrain_gb300._alg3d import Backprop3D

    sino, angles = ellipsoid_phantom_sinogram(48, 24, seed=31,
                                              count_range=(2, 4),
                                              semi_range=(4, 12))
    dev = cuda_ready
    # a 16 MiB workspace limit gives several angle batches, so the
    # compensation buffer inside the scratch is exercised too
    rec = Backprop3D(sino.shape, angles, 3.0, 1.333, padfac=1.75,
                     intp_order=2, input_dtype="complex64", device=dev,
                     workspace_limit=16 << 20)
    assert rec.plan.workspace_bytes <= _native.NOALLOC_SCRATCH_BYTES
    assert rec.plan.angle_batch < len(angles)
    d = torch.from_numpy(sino.astype(np.complex64)).to(dev)
    ref = rec(d)  # odt_bpp3d_execute with a caller workspace

    lib = _native.lib()
    stream = torch.cuda.current_stream(dev)
    for call in range(2):
        out = torch.full(rec.volume_shape(), float("nan"), device=dev,
                         dtype=torch.complex64)
        st = lib.odt_bpp3d_execute_noalloc(
            rec.plan._h, ctypes.c_void_p(d.data_ptr()),
            ctypes.c_void_p(rec.weights.data_ptr()),
            ctypes.c_void_p(rec.geometry.data_ptr()),
            ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(stream.cuda_stream))
        _native.check(st)
        rec.check()
        ok, rel, mx = _close(out, ref)
        assert ok, "call %d: rel-L2 %.3e, max %.3e" % (call, rel, mx)


def test_noalloc_rejects_large_plans(cuda_ready):
    import torch
    from odtbrain_gb300 import _native
    from odtbrain_gb300._alg3d import Backprop3D

    sino, angles = ellipsoid_phantom_sinogram(48, 24, seed=32,
                                              count_range=(2, 4),
                                              semi_range=(4, 12))
    dev = cuda_ready
    rec = Backprop3D(sino.shape, angles, 3.0, 1.333,
                     input_dtype="complex64", device=dev)
    assert rec.plan.workspace_bytes > _native.NOALLOC_SCRATCH_BYTES
    d = torch.from_numpy(sino.astype(np.complex64)).to(dev)
    out = torch.empty(rec.volume_shape(), device=dev, dtype=torch.complex64)
    st = _native.lib().odt_bpp3d_execute_noalloc(
        rec.plan._h, ctypes.c_void_p(d.data_ptr()),
        ctypes.c_void_p(rec.weights.data_ptr()),
        ctypes.c_void_p(rec.geometry.data_ptr()),
        ctypes.c_void_p(out.data_ptr()),
        ctypes.c_void_p(torch.cuda.current_stream(dev).cuda_stream))
    assert st == _native.ODT_ERR_INVALID_ARGUMENT
    assert b"workspace_limit" in _native.lib().odt_last_error()
