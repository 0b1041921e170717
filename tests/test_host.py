"""CPU tests of the host side: FP64 geometry bit-identical to the
reference's, input validation and error types, and the C ABI library (it
loads and exports every symbol include/odtbrain_gb300.h declares; its
argument checks run without a GPU)."""
import ctypes
import os
import re

import numpy as np
import pytest

import odtbrain_gb300 as odt
from odtbrain_gb300 import _geometry as geom
from odtbrain_gb300 import _native, build

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def test_weights_bit_identical(golden):
    g = golden["reference_geometry"]
    keys = [k for k in g if k.startswith("weights_") and
            k.endswith("__angles")]
    assert keys
    for k in keys:
        stem = k[:-len("__angles")]
        assert np.array_equal(geom.compute_angle_weights_1d(g[k]),
                              g[stem + "__w"]), stem


def test_tilted_geometry_bit_identical(golden):
    g = golden["reference_geometry"]
    for i in range(4):
        axis = g["tilt%d__axis" % i]
        angles = g["tilt%d__angles" % i]
        axis_n = geom.norm_vec(axis)
        angz = np.arctan2(axis_n[0], axis_n[1])
        rotmat = np.array([[np.cos(angz), -np.sin(angz), 0],
                           [np.sin(angz), np.cos(angz), 0], [0, 0, 1]])
        axis_yz = geom.norm_vec(np.dot(rotmat, axis_n))
        pts = geom.sphere_points_from_angles_and_tilt(angles, axis_yz)
        assert np.array_equal(pts, g["tilt%d__points" % i])
        _w, mats, _ax = geom.tilted_geometry(angles, axis, False,
                                             (30, 24, 30))
        assert np.array_equal(mats, g["tilt%d__geo" % i]), i


def test_sphere_points_known_answers():
    """test_spherecoords_from_angles_and_axis.py:8-30."""
    angles = np.array([0, np.pi / 2, np.pi])
    axes = [[1, 0, 0], [0, 1, 0], [0, 0, 1], [0, 1, 1], [1, 0, 1], [1, 1, 1]]
    s2 = 1 / np.sqrt(2)
    correct = np.array([[[1, 0, 0], [1, 0, 0], [1, 0, 0]],
                        [[0, 0, 1], [1, 0, 0], [0, 0, -1]],
                        [[0, 0, 1], [0, 0, 1], [0, 0, 1]],
                        [[0, 0, 1], [s2, .5, .5], [0, 1, 0]],
                        [[s2, 0, s2], [s2, 0, s2], [s2, 0, s2]],
                        [[s2, 0, s2],
                         [0.87965281125489458, s2 / 3 * 2,
                          0.063156230327168605],
                         [s2 / 3, s2 / 3 * 4, s2 / 3]]])
    res = [geom.sphere_points_from_angles_and_tilt(angles, ax)
           for ax in axes]
    assert np.allclose(correct, np.array(res))


def test_rotation_matrices_known_answers():
    """test_rotation_matrices.py:8-102."""
    sq2 = np.sqrt(2)
    rot = geom.rotate_points_to_axis(points=[[1, 2, 3]], axis=[1, 2, 3])
    assert rot[0][0] < 1e-14 and rot[0][2] < 1e-14
    rot = geom.rotate_points_to_axis(points=[[0, 0, 1], [1, 0, 0], [1, 1, 0]],
                                     axis=[0, 1, 1])
    assert np.allclose(rot[0], [0, 1 / sq2, 1 / sq2])
    assert np.allclose(rot[1], [1, 0, 0])
    assert np.allclose(rot[2], [1, 1 / sq2, -1 / sq2])
    rot = geom.rotate_points_to_axis(points=[[0, 0, 1], [1, 0, 0],
                                             [0, -1, 0]], axis=[1, 0, 1])
    assert np.allclose(rot[0], [-.5, 1 / sq2, .5])
    assert np.allclose(rot[1], [.5, 1 / sq2, -.5])
    assert np.allclose(rot[2], [1 / sq2, 0, 1 / sq2])
    rot = geom.rotate_points_to_axis(points=[[0, 0, 1], [1, 0, 0],
                                             [1, -1, 0]], axis=[0, -1, 0])
    assert np.allclose(rot[0], [0, 0, -1])
    m1 = geom.rotation_matrix_from_point([0, 0, 1])
    assert np.allclose(np.dot(m1, [1, 2, 3]), [1, 2, 3])
    m2 = geom.rotation_matrix_from_point([0, 1, 1])
    assert np.allclose(np.dot(m2, [0, 0, 1]), [0, 1 / sq2, 1 / sq2])
    m3 = geom.rotation_matrix_from_point([-1, 1, 0])
    assert np.allclose(np.dot(m3, [1, 0, 0]), [0, 0, -1])
    assert np.allclose(np.dot(m3, [0, 1 / sq2, -1 / sq2]), [-1, 0, 0])


def test_rotation_y_geometry_matches_scipy_construction():
    from scipy import special
    angles = np.linspace(0, 2 * np.pi, 200, endpoint=False)
    g = geom.rotation_y_geometry(angles, 256, 256)
    for i in (0, 50, 77, 199):
        deg = -np.rad2deg(angles[i])
        c, s = special.cosdg(deg), special.sindg(deg)
        R = np.array([[c, s], [-s, c]])
        shp = np.asarray((256, 256))
        off = (shp - 1) / 2 - R @ ((shp - 1) / 2)
        assert np.array_equal(g[i, :4], R.reshape(-1))
        assert np.array_equal(g[i, 4:], off)


def test_padding_geometry():
    g = geom.padding_geometry(256, 256, (True, True), 1.75)
    assert (g["lNx"], g["lNy"], g["padxl"], g["padyl"]) == (512, 512, 128,
                                                            128)
    g = geom.padding_geometry(200, 200, (True, True), 1.75)
    assert (g["lNx"], g["padxl"], g["padxr"]) == (512, 156, 156)
    g = geom.padding_geometry(22, 22, (True, True), 1.75)
    assert g["lNx"] == 64
    g = geom.padding_geometry(128, 128, (True, True), 1.75)
    assert g["lNx"] == 256
    g = geom.padding_geometry(22, 17, (False, False), 1.75)
    assert (g["lNx"], g["lNy"]) == (17, 22)


@pytest.mark.parametrize("kwargs,exc", [
    (dict(padding=(True,)), ValueError),
    (dict(padding=(1, 1)), ValueError),
    (dict(padding=(True, False)), ValueError),
    (dict(coords=np.zeros((3, 4))), NotImplementedError),
    (dict(num_cores=10 ** 6), ValueError),
    (dict(dtype=np.int32), ValueError),
])
@pytest.mark.parametrize("fn", ["backpropagate_3d", "backpropagate_3d_tilted"])
def test_validation_errors(fn, kwargs, exc):
    sino = np.ones((4, 8, 8), dtype=complex)
    angles = np.linspace(0, np.pi, 4)
    with pytest.raises(exc):
        getattr(odt, fn)(sino, angles, 3.0, 1.333, **kwargs)


def test_shape_errors():
    with pytest.raises(ValueError):
        odt.backpropagate_3d(np.ones((4, 8), complex), np.zeros(4), 3, 1.3)
    with pytest.raises(ValueError):
        odt.backpropagate_3d(np.ones((4, 8, 8), complex), np.zeros(3), 3,
                             1.3)
    with pytest.raises(ValueError):
        odt.backpropagate_3d_tilted(np.ones((4, 8, 8), complex),
                                    np.zeros((4, 2)), 3, 1.3)


def _header_symbols():
    text = open(os.path.join(ROOT, "include", "odtbrain_gb300.h")).read()
    return sorted(set(re.findall(r"\b(odt_[a-z0-9_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def native_lib():
    build.build()
    return _native.lib()


def test_library_exports_every_declared_symbol(native_lib):
    declared = _header_symbols()
    assert set(declared) == set(_native.EXPORTED_SYMBOLS)
    for name in declared:
        assert hasattr(native_lib, name), name


def test_plan_create_argument_checks(native_lib):
    """Validation happens before any CUDA call, so it runs on CPU."""
    d = _native.Bpp3dDesc()
    d.num_angles, d.ny, d.nx = 4, 16, 16
    d.pad_ny = d.pad_nx = 64
    d.pad_y_left = d.pad_x_left = 24
    d.pad_mode = _native.ODT_PAD_EDGE
    d.intp_order = 6
    filt = np.zeros(64 * 64 * 2)
    ph = np.zeros(64 * 64)
    d.filter = filt.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.kz_phase = ph.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    h = ctypes.c_void_p()
    st = native_lib.odt_bpp3d_plan_create(ctypes.byref(d), ctypes.byref(h))
    assert st == _native.ODT_ERR_INVALID_ARGUMENT
    assert b"0..5" in native_lib.odt_last_error()
    # orders 4 and 5 (two prefilter poles) need lines of >= 4 samples
    d.intp_order = 5
    d.nx = 3
    d.pad_nx = 3
    d.pad_x_left = 0
    st = native_lib.odt_bpp3d_plan_create(ctypes.byref(d), ctypes.byref(h))
    assert st == _native.ODT_ERR_UNSUPPORTED
    with pytest.raises(NotImplementedError):
        _native.check(st)
    d.nx, d.pad_nx, d.pad_x_left = 16, 64, 24
    d.intp_order = 2
    d.pad_x_left = 60
    st = native_lib.odt_bpp3d_plan_create(ctypes.byref(d), ctypes.byref(h))
    assert st == _native.ODT_ERR_INVALID_ARGUMENT
    assert b"padding" in native_lib.odt_last_error()
    d.pad_x_left = 24
    d.pad_nx = 3000  # neither a supported power of two nor <= 1024
    st = native_lib.odt_bpp3d_plan_create(ctypes.byref(d), ctypes.byref(h))
    assert st == _native.ODT_ERR_UNSUPPORTED
    assert native_lib.odt_status_string(5) == b"device-side check failed"


def _sino_desc(A=3, ny=8, nx=9, dtype=None, kind=None, align=1):
    d = _native.SinoDesc()
    d.num_angles, d.ny, d.nx = A, ny, nx
    d.dtype = _native.ODT_DATA_C64 if dtype is None else dtype
    d.kind = _native.ODT_SINO_RYTOV if kind is None else kind
    d.align = align
    d.seed = 47
    d.u0_re = 1.0
    return d


def test_sino_descriptor_checks(native_lib):
    """odt_sino_workspace_size validates the descriptor on the host."""
    nb = ctypes.c_uint64()
    ok = native_lib.odt_sino_workspace_size
    assert ok(ctypes.byref(_sino_desc()), ctypes.byref(nb)) == _native.ODT_OK
    three_d = nb.value
    assert ok(ctypes.byref(_sino_desc(ny=0)), ctypes.byref(nb)) == _native.ODT_OK
    assert 0 < nb.value < three_d  # no spanning-tree buffers for lines
    for bad in (_sino_desc(A=0), _sino_desc(nx=0), _sino_desc(ny=-1),
                _sino_desc(dtype=_native.ODT_DATA_F32),
                _sino_desc(kind=7), _sino_desc(ny=0, nx=2),
                _sino_desc(kind=_native.ODT_SINO_ALIGN),
                _sino_desc(kind=_native.ODT_SINO_ALIGN,
                           dtype=_native.ODT_DATA_F64, align=0),
                _sino_desc(A=70000, ny=2, nx=2)):
        assert ok(ctypes.byref(bad), ctypes.byref(nb)) == \
            _native.ODT_ERR_INVALID_ARGUMENT
    real = _sino_desc(kind=_native.ODT_SINO_UNWRAP, dtype=_native.ODT_DATA_F64)
    assert ok(ctypes.byref(real), ctypes.byref(nb)) == _native.ODT_OK
    n = ctypes.c_int32()
    assert native_lib.odt_sino_launch_count(
        ctypes.byref(_sino_desc()), ctypes.byref(n)) == _native.ODT_OK
    assert n.value > 20
    assert native_lib.odt_sino_prepare(
        ctypes.byref(_sino_desc()), None, None, None, 0, None) == \
        _native.ODT_ERR_INVALID_ARGUMENT


def test_apple_descriptor_checks(native_lib):
    """odt_apple_workspace_size validates the descriptor on the host."""
    from odtbrain_gb300 import apple
    nb = ctypes.c_uint64()
    ws = native_lib.odt_apple_workspace_size
    d = apple._desc((16, 12, 16), 2.1, 1.333)
    assert ws(ctypes.byref(d), ctypes.byref(nb)) == _native.ODT_OK
    with_env = nb.value
    d = apple._desc((16, 12, 16), 2.1, 1.333, enforce_envelope=0)
    assert ws(ctypes.byref(d), ctypes.byref(nb)) == _native.ODT_OK
    assert nb.value < with_env  # no envelope buffers
    for shape, kw, code in [
            ((16, 12, 15), {}, _native.ODT_ERR_INVALID_ARGUMENT),
            ((16, 12, 16), {"enforce_envelope": 1.2},
             _native.ODT_ERR_INVALID_ARGUMENT),
            ((16, 12, 16), {"max_iter": -1}, _native.ODT_ERR_INVALID_ARGUMENT),
            ((1500, 8, 1500), {}, _native.ODT_ERR_UNSUPPORTED)]:
        d = apple._desc(shape, 2.1, 1.333, **kw)
        assert ws(ctypes.byref(d), ctypes.byref(nb)) == code, (shape, kw)
    # another method name: no constraint (the reference's loop then runs
    # without one)
    d = apple._desc((16, 12, 16), 2.1, 1.333, method="other")
    assert d.method == _native.ODT_APPLE_NONE
    assert ws(ctypes.byref(d), ctypes.byref(nb)) == _native.ODT_OK


def test_apple_helper_argument_checks(native_lib):
    """odt_apple_constrain / odt_apple_envelope check their arguments on the
    host before anything is launched (no device pointer is touched)."""
    from odtbrain_gb300 import apple
    nb = ctypes.c_uint64()
    d = _native.AppleDesc()
    d.n0, d.n1, d.n2 = 12, 20, 9  # any 3D shape for a constraint
    d.method = _native.ODT_APPLE_SH
    assert native_lib.odt_apple_constrain_workspace_size(
        ctypes.byref(d), ctypes.byref(nb)) == _native.ODT_OK
    assert nb.value >= 12 * 20 * 9
    bad = _native.ODT_ERR_INVALID_ARGUMENT
    fake = ctypes.c_void_p(4096)  # never dereferenced: the checks fail first
    con = native_lib.odt_apple_constrain
    assert con(ctypes.byref(d), 16, 1, fake, None, None, fake, nb.value,
               None) == bad  # real_bits
    assert con(ctypes.byref(d), 32, 2, fake, None, None, fake, nb.value,
               None) == bad  # is_complex
    assert con(ctypes.byref(d), 32, 1, None, None, None, fake, nb.value,
               None) == bad  # data
    assert con(ctypes.byref(d), 32, 1, fake, None, None, fake, nb.value - 1,
               None) == bad  # workspace size
    assert con(ctypes.byref(d), 64, 0, ctypes.c_void_p(4100), None, None,
               fake, nb.value, None) == bad  # alignment
    d.method = _native.ODT_APPLE_NONE
    assert con(ctypes.byref(d), 32, 1, fake, None, None, fake, nb.value,
               None) == bad  # method
    e = apple._desc((16, 12, 16), 2.1, 1.333)
    assert native_lib.odt_apple_envelope_workspace_size(
        ctypes.byref(e), ctypes.byref(nb)) == _native.ODT_OK
    env = native_lib.odt_apple_envelope
    assert env(ctypes.byref(e), 32, fake, None, fake, fake, nb.value,
               None) == bad  # core
    assert env(ctypes.byref(e), 64, ctypes.c_void_p(4104), fake, fake, fake,
               nb.value, None) == bad  # complex128 alignment
    e = apple._desc((16, 12, 15), 2.1, 1.333)
    assert native_lib.odt_apple_envelope_workspace_size(
        ctypes.byref(e), ctypes.byref(nb)) == bad  # n0 != n2
    e = apple._desc((16, 12, 16), 2.1, 1.333)
    e.gauss_radius = 65
    assert native_lib.odt_apple_envelope_workspace_size(
        ctypes.byref(e), ctypes.byref(nb)) == _native.ODT_ERR_UNSUPPORTED


def test_apple_helper_dtype_errors():
    """The Python drop-ins refuse what the kernels do not compute, before
    touching a device."""
    from odtbrain_gb300 import apple
    with pytest.raises(TypeError):
        apple.constraint_nn(np.zeros((4, 4, 4), dtype=np.int32))
    with pytest.raises(ValueError):
        apple.constraint_sh(np.zeros((4, 4), dtype=np.float32))
    with pytest.raises(ValueError):
        apple.envelope_gauss(np.zeros((4, 5, 6), dtype=np.complex64),
                             np.zeros((4, 5, 6), dtype=bool))


def test_apple_gauss_weights_match_scipy():
    """The 1D Gaussian handed to the envelope kernel is scipy's."""
    import scipy.ndimage as ndi
    from odtbrain_gb300 import apple
    for shape in ((10, 10, 10), (64, 40, 64), (256, 256, 256)):
        w, r = apple._gauss_weights(shape)
        sigma = max(shape) / 100
        x = np.zeros(2 * r + 9)
        x[r + 4] = 1.0
        ref = ndi.gaussian_filter1d(x, sigma, mode="constant", truncate=4.0)
        np.testing.assert_array_equal(ref[4:4 + 2 * r + 1], w[::-1])


def test_public_names_match_the_reference():
    """The package exposes the reference's public names
    (odtbrain/__init__.py:3-15) for the paths it implements; the 2D
    Fourier-mapping and direct-integration algorithms are not built."""
    for name in ("backpropagate_2d", "backpropagate_3d",
                 "backpropagate_3d_tilted", "sinogram_as_radon",
                 "sinogram_as_rytov", "odt_to_ri", "opt_to_ri", "apple",
                 "util", "warn", "__version__"):
        assert hasattr(odt, name), name
    for name in ("apple_core_3d", "correct", "spillover_region",
                 "ellipsoid_shell", "count_to_half", "constraint_nn",
                 "constraint_sh", "envelope_gauss"):
        assert callable(getattr(odt.apple, name)), name
    assert callable(odt.util.compute_angle_weights_1d)
    assert issubclass(odt.warn.DataUndersampledWarning, UserWarning)
    assert issubclass(odt.warn.ImplementationAmbiguousWarning, UserWarning)


def _small_desc(d_arrays):
    d = _native.Bpp3dDesc()
    d.num_angles, d.ny, d.nx = 4, 16, 16
    d.pad_ny = d.pad_nx = 64
    d.pad_y_left = d.pad_x_left = 24
    d.pad_mode = _native.ODT_PAD_EDGE
    d.intp_order = 2
    filt = np.zeros(64 * 64 * 2)
    ph = np.zeros(64 * 64)
    d_arrays.extend([filt, ph])
    d.filter = filt.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    d.kz_phase = ph.ctypes.data_as(ctypes.POINTER(ctypes.c_double))
    return d


def test_forced_allocation_failure_raises_memory_error(native_lib):
    """A plan whose device tables exceed the injected allocation limit is
    refused with ODT_ERR_OUT_OF_MEMORY before any CUDA call (so this runs on
    CPU), and the Python binding turns that into MemoryError."""
    keep = []
    d = _small_desc(keep)
    h = ctypes.c_void_p()
    _native.set_table_alloc_limit(1024)
    try:
        st = native_lib.odt_bpp3d_plan_create(ctypes.byref(d), ctypes.byref(h))
        assert st == _native.ODT_ERR_OUT_OF_MEMORY
        assert not h.value
        assert b"allocation limit" in native_lib.odt_last_error()
        with pytest.raises(MemoryError, match="allocation limit"):
            _native.Plan(d)
    finally:
        _native.set_table_alloc_limit(0)
    # validation still comes first: a bad descriptor stays a ValueError
    d.pad_x_left = 60
    _native.set_table_alloc_limit(1024)
    try:
        with pytest.raises(ValueError, match="padding"):
            _native.Plan(d)
    finally:
        _native.set_table_alloc_limit(0)


def test_slab_size_limit(native_lib):
    """One angle's coefficient slab is addressed with 32-bit element
    offsets: a plan whose slab would hold 2^31 elements or more is refused
    as unsupported before any device call."""
    keep = []
    d = _small_desc(keep)
    d.ny, d.nx = 1024, 2048          # 2048 * 2048 * 1024 = 2^32 elements
    d.pad_ny, d.pad_nx = 2048, 4096
    d.pad_y_left, d.pad_x_left = 512, 1024
    h = ctypes.c_void_p()
    st = native_lib.odt_bpp3d_plan_create(ctypes.byref(d), ctypes.byref(h))
    assert st == _native.ODT_ERR_UNSUPPORTED and not h.value
    assert b"2^31" in native_lib.odt_last_error()


def test_mlp_kernel_selection_argument_check(native_lib):
    """odt_mlp_select_kernels takes 0 (warp-level mma.sync) or 1 (tcgen05)
    and refuses anything else without touching a device."""
    assert native_lib.odt_mlp_select_kernels(2) == _native.ODT_ERR_INVALID_ARGUMENT
    assert b"tensor_memory" in native_lib.odt_last_error()
    assert native_lib.odt_mlp_select_kernels(-1) == _native.ODT_ERR_INVALID_ARGUMENT
    assert native_lib.odt_mlp_select_kernels(0) == 0
    assert native_lib.odt_mlp_select_kernels(1) == 0


def test_status_codes_map_to_python_exceptions(native_lib):
    """Each non-OK status becomes the exception the reference's callers
    expect (ValueError / NotImplementedError / MemoryError) or OdtError."""
    expect = {_native.ODT_ERR_INVALID_ARGUMENT: ValueError,
              _native.ODT_ERR_UNSUPPORTED: NotImplementedError,
              _native.ODT_ERR_OUT_OF_MEMORY: MemoryError,
              _native.ODT_ERR_CUDA: _native.OdtError,
              _native.ODT_ERR_DEVICE_CHECK: _native.OdtError}
    for st, exc in expect.items():
        with pytest.raises(exc) as info:
            _native.check(st)
        if exc is _native.OdtError:
            assert info.value.status == st
    _native.check(_native.ODT_OK)
