"""GPU tests of the learned filter gain.

* the BF16 tensor-core MLP kernels (odt_mlp_gain_forward / _backward)
  against the CPU oracle (oracle/mlp_oracle.py) with the same BF16 operand
  rounding, at ragged sizes (point counts that are not multiples of the
  16-point tile);
* the chain used in training: reconstruction adjoint -> gain gradient ->
  MLP parameter gradients, against central differences of the loss in the
  output bias (FP32 in the kernels, so the perturbation is exact);
* a short training run on a small wedge: the learned gain beats the plain
  filter on held-out phantoms, and the plain filter stays available as the
  fallback.
"""
import numpy as np
import pytest

from oracle import mlp_oracle as M

pytestmark = pytest.mark.gpu


def _rel(a, b):
    return np.linalg.norm(np.asarray(a) - np.asarray(b)) / \
        np.linalg.norm(np.asarray(b))


def _random_mlp(torch, dev, seed, scale=1.0):
    from odtbrain_gb300.learned import GainMLP, PARAM_SHAPES
    rng = np.random.default_rng(seed)
    st = {}
    for k, shape in PARAM_SHAPES.items():
        fan = shape[1] if len(shape) == 2 else 64
        st[k] = rng.normal(0, scale / np.sqrt(fan), shape).astype(np.float32)
    m = GainMLP(device=dev)
    m.load_state(st)
    return m, st


@pytest.mark.parametrize("A,lNy,lNx", [(3, 32, 32), (2, 17, 30), (1, 5, 3)])
def test_mlp_forward_matches_oracle(cuda_ready, A, lNy, lNx):
    import torch
    dev = cuda_ready
    m, st = _random_mlp(torch, dev, seed=A + lNx)
    rng = np.random.default_rng(7)
    af = rng.uniform(-1.5, 1.5, (A, 2)).astype(np.float32)
    g = m.gains(torch.tensor(af, device=dev), lNy, lNx).cpu().numpy()
    m.check()  # no tensor-core completion wait gave up
    X = M.features(af, lNy, lNx)
    ref, _ = M.forward(st, X, bf16=True)
    exact, _ = M.forward(st, X, bf16=False)
    got = g.reshape(-1)
    assert np.all(np.isfinite(got))
    assert _rel(got - 1, ref - 1) < 1e-3
    # BF16 operands against the exact FP64 network
    assert _rel(got - 1, exact - 1) < 5e-2


def test_mlp_forward_many_tiles(cuda_ready):
    """262,144 points: more 128-point tiles than the persistent grid has
    warp groups, so every group carries several tiles through the
    tensor-memory accumulators, twice in a row."""
    import torch
    dev = cuda_ready
    m, st = _random_mlp(torch, dev, seed=5)
    rng = np.random.default_rng(9)
    A, lNy, lNx = 4, 256, 256
    af = rng.uniform(-1.5, 1.5, (A, 2)).astype(np.float32)
    X = M.features(af, lNy, lNx)
    ref, _ = M.forward(st, X, bf16=True)
    for _ in range(2):
        got = m.gains(torch.tensor(af, device=dev), lNy, lNx).cpu().numpy()
        m.check()
        got = got.reshape(-1)
        assert np.all(np.isfinite(got))
        assert _rel(got - 1, ref - 1) < 1e-3


@pytest.mark.parametrize("A,lNy,lNx", [(3, 32, 32), (2, 17, 30)])
def test_mlp_backward_matches_oracle(cuda_ready, A, lNy, lNx):
    import torch
    dev = cuda_ready
    m, st = _random_mlp(torch, dev, seed=11 + A)
    rng = np.random.default_rng(8)
    af = rng.uniform(-1.5, 1.5, (A, 2)).astype(np.float32)
    dg = (rng.normal(size=(A, lNy, lNx)) +
          1j * rng.normal(size=(A, lNy, lNx))).astype(np.complex64)
    grads = m.grads(torch.tensor(af, device=dev), torch.tensor(dg,
                                                             device=dev))
    X = M.features(af, lNy, lNx)
    ref = M.backward(st, X, dg.reshape(-1), bf16=True)
    exact = M.backward(st, X, dg.reshape(-1), bf16=False)
    for k in ref:
        got = grads[k].cpu().numpy()
        assert got.shape == ref[k].shape, k
        assert _rel(got, ref[k]) < 2e-3, k
        assert _rel(got, exact[k]) < 5e-2, k


def test_mlp_positions(cuda_ready):
    """A position list evaluates only the listed entries (others keep their
    value) and restricts the backward to them."""
    import torch
    dev = cuda_ready
    m, st = _random_mlp(torch, dev, seed=3)
    A, lNy, lNx = 3, 20, 24
    rng = np.random.default_rng(9)
    pos = np.sort(rng.choice(lNy * lNx, size=157, replace=False)).astype(
        np.int32)
    af = rng.uniform(-1, 1, (A, 2)).astype(np.float32)
    fd = torch.tensor(af, device=dev)
    full = m.gains(fd, lNy, lNx).cpu().numpy().reshape(A, -1)
    part = m.gains(fd, lNy, lNx, positions=pos).cpu().numpy().reshape(A, -1)
    mask = np.zeros(lNy * lNx, bool)
    mask[pos] = True
    assert np.all(part[:, ~mask] == 1)
    np.testing.assert_array_equal(part[:, mask], full[:, mask])
    dg = (rng.normal(size=(A, lNy * lNx)) +
          1j * rng.normal(size=(A, lNy * lNx))).astype(np.complex64)
    dg[:, ~mask] = 0
    dgt = torch.tensor(dg.reshape(A, lNy, lNx), device=dev)
    g_full = m.grads(fd, dgt)
    g_part = m.grads(fd, dgt, positions=torch.tensor(pos, device=dev))
    for k in g_full:
        a, b = g_part[k].cpu().numpy(), g_full[k].cpu().numpy()
        assert _rel(a, b) < 1e-5, k


def test_training_chain_matches_finite_differences(cuda_ready):
    """d loss / d b4 through the reconstruction adjoint and the MLP
    backward, against central differences of the FP32 forward."""
    import torch
    from odtbrain_gb300._alg3d import Backprop3D
    from odtbrain_gb300.learned import LearnedFilter, wedge_angles
    from odtbrain_gb300 import phantoms
    dev = cuda_ready
    n, A = 24, 10
    angles = wedge_angles(A, 2 * np.pi / 3)
    rec = Backprop3D((A, n, n), angles, 3.0, 1.333, input_dtype="complex64",
                     device=dev)
    m, st = _random_mlp(torch, dev, seed=5, scale=0.5)
    lf = LearnedFilter(rec, m)
    rng = np.random.default_rng(4)
    ells = phantoms.random_ellipsoids(rng, n, (2, 4), (3, 8))
    sino = phantoms.project([ells], angles, n, amp_sigma=0.01, seed=1,
                            device=dev)[0].contiguous()
    tgt = torch.tensor((rng.normal(size=(n, n, n)) +
                        1j * rng.normal(size=(n, n, n))).astype(np.complex64),
                       device=dev) * 0.01

    def loss():
        v = lf(sino).to(torch.complex128) - tgt.to(torch.complex128)
        return (v.abs() ** 2).sum().item()

    vol = lf(sino)
    cot = (2 * (vol - tgt)).to(torch.complex64)
    _s, _g, dgain = rec.adjoint(sino, cot, angle_gain=lf.gains(),
                                need_sino=False, need_angle_gain=True)
    g = m.grads(lf.feat, dgain, positions=lf.positions)
    # b4 is FP32 in the kernels: perturb it directly
    for j in range(2):
        h = 1e-2
        base = st["b4"].copy()
        vals = []
        for s in (+1, -1):
            st2 = dict(st)
            st2["b4"] = base.copy()
            st2["b4"][j] += s * h
            m.load_state(st2)
            vals.append(loss())
        m.load_state(st)
        fd = (vals[0] - vals[1]) / (2 * h)
        an = g["b4"][j].item()
        assert abs(fd - an) <= 3e-3 * abs(an) + 2e-5 * vals[0], (j, fd, an)


def test_short_training_beats_plain_filter(cuda_ready):
    from odtbrain_gb300.learned import train_wedge_filter
    lf, rep = train_wedge_filter(dict(
        n=32, num_angles=12, dense_angles=120, count_range=(1, 4),
        semi_range=(3.0, 9.0), n_train=64, n_val=16, n_eval=16, epochs=3,
        batch=4, lr=3e-3), device=cuda_ready, log=lambda *a: None)
    print("\nsmall wedge: eval rel-L2 learned %.4f plain %.4f (%.1f%%)"
          % (rep["eval_rel_l2_learned"], rep["eval_rel_l2_plain"],
             100 * rep["reduction"]))
    assert rep["enabled"]
    assert rep["eval_rel_l2_learned"] < rep["eval_rel_l2_plain"]
    # the fallback is the plain reconstruction
    lf.enabled = False
    import torch
    s = torch.zeros(lf.rec.shape, dtype=torch.complex64,
                    device=cuda_ready)
    s[:, 3, 4] = 1.0
    a = lf(s)
    b = lf.rec(s)
    assert torch.equal(a, b)


def test_shipped_wedge_network_beats_plain_filter(cuda_ready):
    """The committed network (trained on 2000 phantoms) on 12 phantoms from
    the held-out seed range: rel-L2 to the dense plain reconstruction."""
    from odtbrain_gb300._alg3d import Backprop3D
    from odtbrain_gb300.learned import (WEDGE_CONFIG, evaluate,
                                        load_learned_filter, make_pairs,
                                        wedge_angles)
    c = dict(WEDGE_CONFIG)
    n, A = c["n"], c["num_angles"]
    sp = wedge_angles(A, c["span"])
    de = np.linspace(0, 2 * np.pi, c["dense_angles"], endpoint=False)
    rec = Backprop3D((A, n, n), sp, c["res"], c["nm"], device=cuda_ready)
    rec_d = Backprop3D((c["dense_angles"], n, n), de, c["res"], c["nm"],
                       device=cuda_ready)
    seeds = 2_000_000 + np.arange(12)
    s, t = make_pairs(c, seeds, rec, rec_d, sp, de, cuda_ready)
    lf = load_learned_filter(rec)
    assert lf.enabled
    learned, plain = evaluate(lf, s, t)
    print("\nshipped wedge network: rel-L2 learned %.4f plain %.4f (%.1f%%)"
          % (learned, plain, 100 * (1 - learned / plain)))
    assert learned < 0.7 * plain
