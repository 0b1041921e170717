"""CPU tests of the learned filter's host side and of its oracle.

* the MLP oracle's reverse mode against central finite differences (FP64,
  no BF16 rounding), which pins the code the BF16 mode shares;
* the oracle's BF16 rounding against PyTorch's float32 -> bfloat16;
* the angle features and wedge angles;
* the GPU phantom projector (run here on the CPU device) against the
  analytic-projection generator of the test fixtures.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as M


def _params(rng, scale=1.0):
    p = {}
    for k, shape in (("W1", (64, 4)), ("b1", (64,)), ("W2", (64, 64)),
                     ("b2", (64,)), ("W3", (64, 64)), ("b3", (64,)),
                     ("W4", (2, 64)), ("b4", (2,))):
        fan = shape[1] if len(shape) == 2 else 64
        p[k] = rng.normal(0, scale / np.sqrt(fan), shape)
    return p


def test_oracle_gradients_match_finite_differences():
    rng = np.random.default_rng(0)
    p = _params(rng)
    X = M.features(rng.normal(size=(3, 2)), 5, 6)
    dg = rng.normal(size=X.shape[0]) + 1j * rng.normal(size=X.shape[0])

    def loss(q):
        g, _ = M.forward(q, X, bf16=False)
        return np.sum(dg.real * g.real + dg.imag * g.imag)

    grads = M.backward(p, X, dg, bf16=False)
    h = 1e-6
    for k in p:
        flat = p[k].ravel()
        for idx in rng.choice(flat.size, size=min(6, flat.size),
                              replace=False):
            qp = {kk: vv.copy() for kk, vv in p.items()}
            qm = {kk: vv.copy() for kk, vv in p.items()}
            qp[k].ravel()[idx] += h
            qm[k].ravel()[idx] -= h
            fd = (loss(qp) - loss(qm)) / (2 * h)
            an = grads[k].ravel()[idx]
            assert abs(fd - an) <= 1e-6 * (1 + abs(fd)), (k, idx, fd, an)


def test_bf16_round_matches_torch():
    torch = pytest.importorskip("torch")
    rng = np.random.default_rng(1)
    x = np.concatenate([rng.normal(size=10000).astype(np.float32),
                        np.float32([0.0, -0.0, 1.0, 3.0, 1e-30, -7.5e5]),
                        # exact ties of the BF16 grid
                        np.float32([1.0 + 2.0 ** -8, 1.0 + 3 * 2.0 ** -8])])
    ref = torch.tensor(x).to(torch.bfloat16).float().numpy()
    np.testing.assert_array_equal(M.bf16_round(x), ref)


def test_features_layout():
    af = np.array([[0.25, -1.5], [-0.75, 2.0]], dtype=np.float32)
    X = M.features(af, 4, 5).reshape(2, 4, 5, 4)
    np.testing.assert_allclose(X[0, 0, :, 0], [0, .4, .8, -.8, -.4],
                               rtol=1e-6)
    np.testing.assert_allclose(X[1, :, 0, 1], [0, .5, -1, -.5], rtol=1e-6)
    assert np.all(X[1, ..., 2] == np.float32(-0.75))
    assert np.all(X[0, ..., 3] == np.float32(-1.5))


def test_angle_features_and_wedge():
    from odtbrain_gb300.learned import angle_features, wedge_angles
    full = np.linspace(0, 2 * np.pi, 36, endpoint=False)
    f = angle_features(full)
    np.testing.assert_allclose(f[:, 1], 0.0, atol=1e-6)
    np.testing.assert_allclose(f[:, 0], full / np.pi - 1, atol=1e-6)
    w = wedge_angles(40, 2 * np.pi / 3)
    assert w.size == 40
    np.testing.assert_allclose(np.diff(w), (2 * np.pi / 3) / 40)
    np.testing.assert_allclose(w.mean(), 0.0, atol=1e-12)
    fw = angle_features(w)
    # interior: spacing 3 deg against 9 deg for a uniform full circle
    np.testing.assert_allclose(fw[1:-1, 1], np.log(1 / 3), rtol=1e-6)
    # the two ends carry half the missing 240 deg arc
    end = 0.5 * (np.deg2rad(3) + np.deg2rad(243)) * 40 / (2 * np.pi)
    np.testing.assert_allclose(fw[[0, -1], 1], np.log(end), rtol=1e-6)
    # order does not matter
    perm = np.random.default_rng(2).permutation(40)
    np.testing.assert_allclose(angle_features(w[perm]), fw[perm])


def test_projector_matches_fixture_generator():
    torch = pytest.importorskip("torch")
    from odtbrain_gb300 import phantoms
    from sino_gen import ellipsoid_phantom_sinogram
    n, A = 24, 7
    angles = np.linspace(0, 2 * np.pi, A, endpoint=False) + 0.1
    ref, _ = ellipsoid_phantom_sinogram(n, A, seed=3, count_range=(2, 4),
                                        semi_range=(2, 6), amp_sigma=0.0,
                                        angles=angles)
    rng = np.random.default_rng(3)
    ells = phantoms.random_ellipsoids(rng, n, (2, 4), (2, 6))
    got = phantoms.project([ells], angles, n, device="cpu")[0].numpy()
    assert np.abs(ref.real).max() == 0
    err = np.abs(got.imag - ref.imag).max() / np.abs(ref.imag).max()
    assert err < 1e-4
