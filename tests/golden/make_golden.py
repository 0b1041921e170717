"""Generate the golden fixtures in ``tests/golden/`` from the unmodified
ODTbrain reference.

Run where the reference source tree is mounted, naming it in
$ODT_REFERENCE_ROOT (the directory that contains ``odtbrain/``):

    ODT_REFERENCE_ROOT=/path/to/ODTbrain python tests/golden/make_golden.py

Writes
  reference_zips.npz   the reference's own golden vectors
                       (tests/data/alg3d_bpp__test_3d_backprop_phase.zip,
                       ..._nopadreal.zip, ..._mprotate.zip,
                       alg2d_bpp__test_2d_backprop_{phase,full}.zip,
                       processing__test_{odt,opt}_to_ri.zip), parsed
  reference_cases.npz  inputs and FP64 outputs of backpropagate_3d /
                       backpropagate_3d_tilted / backpropagate_2d for small
                       cases, produced by
                       the reference itself (through the import shims of
                       refshim.py: scipy.fft for FFTW, NumPy for numexpr)
  reference_geometry.npz  FP64 host geometry of the reference (angle weights,
                       sphere points, rotation matrices, offsets) for
                       bit-exact comparison
  reference_sino.npz   sinogram preparation: the reference's golden
                       vectors (processing__test_sino_{rytov,radon}.zip,
                       apple__test_correct_reproduce.zip) and outputs of its
                       sinogram_as_rytov / sinogram_as_radon

  reference_apple.npz  inputs and outputs of the reference's apple.correct
  reference_apple_helpers.npz  inputs and outputs of the reference's
                       constraint_nn, constraint_sh and envelope_gauss
                       called on their own
  reference_c1.npz     the reference's backpropagate_3d of the whole
                       60-angle, 64x64 -> 64^3 ellipsoid-phantom workload
                       (FP64 run, stored as float32 real/imaginary parts),
                       with a checksum of the regenerated input

Parts can be chosen on the command line (backprop, sino, apple,
apple_helpers, c1); default all.
The input sinogram generator below restates the reference's test helper
(tests/common_methods.py:63-184) so that the GPU tests can regenerate the
same inputs without the reference tree.
"""
import io
import json
import os
import sys
import zipfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, HERE)
sys.path.insert(0, os.path.dirname(HERE))
sys.path.insert(0, os.path.dirname(os.path.dirname(HERE)))

import refshim  # noqa: E402
from sino_gen import gauss_sino_2d, gauss_sino_3d, gauss_sino_3d_tilted, parameter_sets  # noqa: E402,E501


def _read_zip(path):
    with zipfile.ZipFile(path) as z:
        return np.loadtxt(io.BytesIO(z.read("data.txt")))


def main(parts):
    odt = refshim.load_reference()
    if "backprop" in parts:
        make_backprop(odt)
    if "sino" in parts:
        make_sino(odt)
    if "apple" in parts:
        make_apple(odt)
    if "apple_helpers" in parts:
        make_apple_helpers(odt)
    if "c1" in parts:
        make_c1(odt)
    print("wrote fixtures to", HERE)


# The 60-angle 64^3 workload: seeded ellipsoid phantom (1-5 ellipsoids,
# semi-axes 5-20 px), padfac 1.75 (128^2 FFTs), intp_order 2, complex
# output, angle weights on.  tests/test_gpu_parity.py regenerates the input
# with the same call.
C1_ARGS = dict(n=64, A=60, seed=2023, count_range=(1, 5), semi_range=(5, 20))
C1_KW = dict(res=3.0, nm=1.333, padfac=1.75, intp_order=2, onlyreal=False)


def make_c1(odt):
    from sino_gen import ellipsoid_phantom_sinogram
    sino, angles = ellipsoid_phantom_sinogram(**C1_ARGS)
    out = odt.backpropagate_3d(sino, angles, **C1_KW)
    np.savez_compressed(
        os.path.join(HERE, "reference_c1.npz"),
        out_re=out.real.astype(np.float32),
        out_im=out.imag.astype(np.float32),
        input_abs_sum=np.abs(sino).sum(), angles=angles,
        kw=np.array(json.dumps(C1_KW)), args=np.array(json.dumps(C1_ARGS)))


def make_backprop(odt):
    from odtbrain import _alg3d_bppt as bppt
    root = refshim.REFERENCE_ROOT
    data = os.path.join(root, "tests", "data")
    zips = {}
    for name in ("test_3d_backprop_phase", "test_3d_backprop_nopadreal",
                 "test_3d_mprotate"):
        zips[name] = _read_zip(os.path.join(data,
                                            "alg3d_bpp__%s.zip" % name))
    for name in ("test_2d_backprop_phase", "test_2d_backprop_full"):
        zips[name] = _read_zip(os.path.join(data,
                                            "alg2d_bpp__%s.zip" % name))
    for name in ("test_odt_to_ri", "test_opt_to_ri"):
        zips[name] = _read_zip(os.path.join(data,
                                            "processing__%s.zip" % name))
    np.savez_compressed(os.path.join(HERE, "reference_zips.npz"), **zips)

    cases = {}

    def add(name, fn, sino, angles, **kw):
        out = fn(sino, angles, **kw)
        cases[name + "__sino"] = sino
        cases[name + "__angles"] = np.asarray(angles)
        cases[name + "__out"] = out
        clean = {}
        for k, v in kw.items():
            if k == "dtype":
                continue  # every case runs at the reference default, float64
            if isinstance(v, (list, tuple)) and k == "tilted_axis":
                v = [float(t) for t in v]
            elif isinstance(v, np.floating):
                v = float(v)
            clean[k] = v
        cases[name + "__kw"] = np.array(json.dumps(clean))

    sino, angles = gauss_sino_3d()
    p1, p2 = parameter_sets(2)
    add("bpp_ramp0_p2", odt.backpropagate_3d, sino, angles, padval=0,
        dtype=float, **p2)
    add("bpp_edge_p1", odt.backpropagate_3d, sino, angles, padval="edge",
        dtype=float, **p1)
    s2, a2 = gauss_sino_3d(A=7, Nx=17, Ny=13, max_phase=3.0,
                          ampl_range=(0.8, 1.1))
    add("bpp_rect_order3", odt.backpropagate_3d, s2, a2, padval="edge",
        intp_order=3, dtype=float, **p1)
    add("bpp_rect_nopad", odt.backpropagate_3d, s2, a2,
        padding=(False, False), dtype=float, **p2)
    # quartic and quintic splines (two prefilter poles)
    add("bpp_order4", odt.backpropagate_3d, sino, angles, padval="edge",
        intp_order=4, dtype=float, **p1)
    add("bpp_rect_order5", odt.backpropagate_3d, s2, a2, padval=0,
        intp_order=5, dtype=float, **p2)
    add("bppt_default_p2", odt.backpropagate_3d_tilted, sino, angles,
        padval=0, dtype=float, **p2)
    st, at = gauss_sino_3d_tilted(A=11, tilt_plane=0.3)
    ax = [np.sin(0.3), np.cos(0.3), 0.15]
    add("bppt_axis_order2", odt.backpropagate_3d_tilted, st, at,
        tilted_axis=ax, padval="edge", dtype=float, **p1)
    add("bppt_axis_order1", odt.backpropagate_3d_tilted, st, at,
        tilted_axis=ax, intp_order=1, padval=0, dtype=float, **p1)
    add("bppt_axis_order5", odt.backpropagate_3d_tilted, st, at,
        tilted_axis=ax, intp_order=5, padval="edge", dtype=float, **p1)
    add("bppt_rect_order4", odt.backpropagate_3d_tilted, s2, a2,
        tilted_axis=[0, np.cos(0.2), np.sin(0.2)], intp_order=4,
        dtype=float, **p2)
    add("bppt_yz_onlyreal", odt.backpropagate_3d_tilted, s2, a2,
        tilted_axis=[0, np.cos(0.2), np.sin(0.2)], onlyreal=True,
        dtype=float, **p2)
    pts = bppt.sphere_points_from_angles_and_tilt(
        at, np.array([0, np.cos(0.4), np.sin(0.4)]))
    add("bppt_points3", odt.backpropagate_3d_tilted, st, pts,
        tilted_axis=[0, np.cos(0.4), np.sin(0.4)], weight_angles=False,
        dtype=float, **p1)
    # 2D path
    s2d, a2d = gauss_sino_2d()
    s2f, _ = gauss_sino_2d(ampl_range=(0.9, 1.1))
    add("b2d_p1", odt.backpropagate_2d, s2d, a2d, **p1)
    add("b2d_full_p2", odt.backpropagate_2d, s2f, a2d, **p2)
    add("b2d_edge_real", odt.backpropagate_2d, s2f, a2d, padval=None,
        onlyreal=True, **p1)
    rng = np.random.default_rng(11)
    a_rand = np.sort(rng.uniform(0, 2 * np.pi, 13))
    s_odd, _ = gauss_sino_2d(A=13, N=31, max_phase=3.0,
                             ampl_range=(0.8, 1.2))
    add("b2d_odd_nopad", odt.backpropagate_2d, s_odd, a_rand,
        padding=False, **p2)
    add("b2d_odd_noweight", odt.backpropagate_2d, s_odd, a_rand,
        weight_angles=False, padval=1.5, **p1)
    np.savez_compressed(os.path.join(HERE, "reference_cases.npz"), **cases)

    geo = {}
    rng = np.random.default_rng(3)
    angle_sets = {
        "uniform": np.linspace(0, 2 * np.pi, 200, endpoint=False),
        "wedge": np.linspace(0, np.deg2rad(120), 40),
        "random": np.sort(rng.uniform(-1, 7, 37)),
        "dupes": np.concatenate([np.zeros(3), np.linspace(0, np.pi, 9)]),
    }
    for k, a in angle_sets.items():
        geo["weights_%s__angles" % k] = a
        geo["weights_%s__w" % k] = odt.util.compute_angle_weights_1d(a)
    for i, axis in enumerate(([0, np.cos(.2), np.sin(.2)], [0.3, 1, 0.1],
                              [0, 1, 0], [1, 0.1, 0.2])):
        a = np.linspace(0, 2 * np.pi, 23, endpoint=False)
        raw_axis = np.asarray(axis, dtype=float)
        axis = bppt.norm_vec(raw_axis)
        angz = np.arctan2(axis[0], axis[1])
        rotmat = np.array([[np.cos(angz), -np.sin(angz), 0],
                           [np.sin(angz), np.cos(angz), 0],
                           [0, 0, 1]])
        axis_yz = bppt.norm_vec(np.dot(rotmat, axis))
        pts = bppt.sphere_points_from_angles_and_tilt(a, axis_yz)
        rpts = bppt.rotate_points_to_axis(points=pts, axis=axis_yz)
        shape = (30, 24, 30)
        c = 0.5 * np.array(shape) - .5
        mats = []
        for pnt in rpts:
            _d, dinv = bppt.rotation_matrix_from_point_planerot(
                pnt, plane_angle=angz, ret_inv=True)
            mats.append(np.concatenate([dinv.reshape(-1),
                                        c - np.dot(dinv, c)]))
        geo["tilt%d__axis" % i] = raw_axis
        geo["tilt%d__angles" % i] = a
        geo["tilt%d__points" % i] = pts
        geo["tilt%d__geo" % i] = np.array(mats)
    np.savez_compressed(os.path.join(HERE, "reference_geometry.npz"), **geo)


def make_sino(odt):
    """reference_sino.npz: the reference's golden vectors of the sinogram
    preparation and of apple.correct (tests/data/processing__test_sino_*.zip,
    apple__test_correct_reproduce.zip), and outputs of the reference's own
    sinogram_as_rytov / sinogram_as_radon.  2D sinograms run the reference
    unmodified (numpy.unwrap); 3D sinograms run it with unwrap_phase
    provided by the oracle's restatement (scikit-image is absent)."""
    from oracle import unwrap_oracle
    data = os.path.join(refshim.REFERENCE_ROOT, "tests", "data")
    out = {}
    for name in ("test_sino_rytov", "test_sino_radon"):
        out["zip_" + name] = _read_zip(os.path.join(
            data, "processing__%s.zip" % name))
    out["zip_test_correct_reproduce"] = _read_zip(os.path.join(
        data, "apple__test_correct_reproduce.zip"))
    refshim.UNWRAP_PHASE[0] = unwrap_oracle.unwrap_2d

    def add(name, kind, sino, u0=None, align=True):
        if kind == "rytov":
            res = (odt.sinogram_as_rytov(sino.copy(), align=align)
                   if u0 is None else
                   odt.sinogram_as_rytov(sino.copy(), u0=u0, align=align))
        else:
            res = odt.sinogram_as_radon(sino.copy(), align=align)
        out[name + "__sino"] = sino
        if u0 is not None:
            out[name + "__u0"] = np.asarray(u0)
        out[name + "__out"] = res
        out[name + "__kw"] = np.array(json.dumps(
            {"kind": kind, "align": bool(align)}))

    s2, _ = gauss_sino_2d(A=13, N=40, max_phase=9.0, ampl_range=(0.7, 1.2))
    add("r2_c128", "rytov", s2)
    add("r2_c128_noalign", "rytov", s2, align=False)
    add("r2_c64", "rytov", s2.astype(np.complex64))
    add("r2_radon", "radon", s2)
    # background phase near pi: the lines start on either side of the cut
    rng = np.random.default_rng(21)
    tilt = np.exp(1j * (np.pi - 0.05 + 0.1 * rng.standard_normal((13, 1))))
    add("r2_nearpi", "rytov", s2 * tilt)
    u0 = 0.9 * np.exp(1j * np.linspace(-0.4, 0.3, 40))
    add("r2_u0_array", "rytov", s2 * u0, u0=u0)
    add("r2_u0_scalar", "rytov", s2 * 2.0, u0=2.0)
    s3, _ = gauss_sino_3d(A=9, Nx=22, Ny=18, max_phase=11.0,
                          ampl_range=(0.8, 1.1))
    add("r3_c128", "rytov", s3)
    add("r3_c128_noalign", "rytov", s3, align=False)
    add("r3_c64", "rytov", s3.astype(np.complex64))
    add("r3_radon", "radon", s3)
    tilt3 = np.exp(1j * (np.pi - 0.02 + 0.05 * rng.standard_normal((9, 1, 1))))
    add("r3_nearpi", "rytov", s3 * tilt3)
    u03 = 1.1 * np.exp(1j * np.linspace(0, 0.5, 22))[None, None, :]
    add("r3_u0_array", "rytov", s3 * u03, u0=u03)
    np.savez_compressed(os.path.join(HERE, "reference_sino.npz"), **out)
    refshim.UNWRAP_PHASE[0] = None


def make_apple(odt):
    """reference_apple.npz: inputs and outputs of the reference's
    apple.correct (odtbrain/apple.py:113-263) for small volumes, run
    unmodified through the pyFFTW stand-in (scipy.fft on complex64 data)."""
    out = {}
    rng = np.random.default_rng(31)

    def volume(A, nx, ny):
        s, a = gauss_sino_3d(A=A, Nx=nx, Ny=ny, max_phase=2.5,
                             ampl_range=(0.9, 1.0))
        # Rytov data of a phase below pi: log of the field
        return odt.backpropagate_3d(np.log(s), a, res=2.5, nm=1.333,
                                    padval=0, dtype=float)

    vols = {"cube": volume(12, 20, 20), "rect": volume(10, 18, 12)}
    for k, v in vols.items():
        out["vol_" + k] = v

    def add(name, vol, **kw):
        f = vols[vol]
        res = odt.apple.correct(f=f.copy(), **kw)
        out[name + "__vol"] = np.array(vol)
        jkw = {k: v for k, v in kw.items() if k != "mask"}
        if "mask" in kw:
            out[name + "__mask"] = kw["mask"]
        out[name + "__kw"] = np.array(json.dumps(jkw))
        out[name + "__out"] = np.asarray(res)

    base = dict(res=2.5, nm=1.333)
    add("nn_default", "cube", **base)
    add("nn_noenvelope", "cube", enforce_envelope=0, **base)
    add("nn_iter5", "cube", max_iter=5, min_diff=0.0, **base)
    add("nn_mask", "cube", mask=rng.random(vols["cube"].shape) > 0.3, **base)
    add("nn_shell", "cube", bg_shell_width=3, **base)
    add("sh_default", "cube", method="sh", **base)
    add("sh_shell", "cube", method="sh", bg_shell_width=3, max_iter=20,
        **base)
    add("nn_rect", "rect", **base)
    add("nn_env50", "cube", enforce_envelope=0.5, min_diff=0.001, **base)
    np.savez_compressed(os.path.join(HERE, "reference_apple.npz"), **out)


def make_apple_helpers(odt):
    """reference_apple_helpers.npz: inputs and outputs of the reference's
    constraint_nn / constraint_sh (odtbrain/apple.py:56-110, in place) and
    envelope_gauss (:289-350), run unmodified on small volumes of float32,
    float64, complex64 and complex128 data."""
    out = {}
    rng = np.random.default_rng(47)

    def volume(A, nx, ny, seed):
        s, a = gauss_sino_3d(A=A, Nx=nx, Ny=ny, max_phase=2.5,
                             ampl_range=(0.9, 1.0))
        s = s * np.exp(0.05j * np.random.default_rng(seed).standard_normal(
            s.shape))
        return odt.backpropagate_3d(np.log(s), a, res=2.5, nm=1.333,
                                    padval=0, dtype=float)

    cube = volume(12, 20, 20, 1)
    rect = volume(10, 18, 12, 2)
    out["in_cube"] = cube
    out["in_rect"] = rect

    def cons(name, fn, src, dtype, mask=None, shell=None):
        # the input is in_<src> cast to dtype (its real part for a real type)
        base = {"cube": cube, "rect": rect}[src]
        if np.issubdtype(dtype, np.complexfloating):
            data = base.astype(dtype)
        else:
            data = np.ascontiguousarray(base.real.astype(dtype))
        kw = {}
        if mask is not None:
            kw["mask"] = mask
            out[name + "__mask"] = mask
        if shell is not None:
            kw["bg_shell"] = shell
            out[name + "__shell"] = shell
        getattr(odt.apple, fn)(data=data, **kw)
        out[name + "__src"] = np.array(src)
        out[name + "__fn"] = np.array(fn)
        out[name + "__out"] = data

    mask_c = rng.random(cube.shape) > 0.3
    mask_r = rng.random(rect.shape) > 0.5
    shell_c = odt.apple.ellipsoid_shell(cube.shape, width=3)
    shell_r = odt.apple.ellipsoid_shell(rect.shape, width=2)
    cons("nn_c64", "constraint_nn", "cube", np.complex64)
    cons("nn_c64_mask_shell", "constraint_nn", "cube", np.complex64,
         mask_c, shell_c)
    cons("nn_f64_shell", "constraint_nn", "cube", np.float64, None, shell_c)
    cons("nn_c128_rect_mask", "constraint_nn", "rect", np.complex128, mask_r)
    cons("sh_c64", "constraint_sh", "cube", np.complex64)
    cons("sh_c64_mask_shell", "constraint_sh", "cube", np.complex64,
         mask_c, shell_c)
    cons("sh_c128", "constraint_sh", "cube", np.complex128)
    cons("sh_f32_rect_shell", "constraint_sh", "rect", np.float32, None,
         shell_r)
    cons("sh_f64_rect_mask", "constraint_sh", "rect", np.float64, mask_r)

    def env(name, src, dtype, res=2.5, nm=1.333):
        ft = np.fft.fftn(src).astype(dtype)
        core = odt.apple.apple_core_3d(shape=src.shape, res=res, nm=nm)
        out[name + "__ft"] = ft
        out[name + "__core"] = core
        out[name + "__out"] = odt.apple.envelope_gauss(ftdata=ft.copy(),
                                                       core=core)

    env("env_c64_cube", cube, np.complex64)
    env("env_c128_cube", cube, np.complex128)
    env("env_c64_rect", rect, np.complex64)  # shape[0] > shape[1]
    tall = np.ascontiguousarray(cube[4:16, :, 4:16])  # shape[0] < shape[1]
    env("env_c64_tall", tall, np.complex64, res=1.5)
    env("env_c128_tall", tall, np.complex128, res=1.5)
    np.savez_compressed(os.path.join(HERE, "reference_apple_helpers.npz"),
                        **out)


if __name__ == "__main__":
    main(sys.argv[1:] or ["backprop", "sino", "apple", "apple_helpers",
                          "c1"])
