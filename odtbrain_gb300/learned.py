"""Learned filter gain for sparse and missing-wedge angle sets.

The reference's backpropagation filter (odtbrain/_alg3d_bpp.py:371-399) is
fixed: |k_x| times the propagator, with angle weights from
odtbrain/util.py:4-67.  For a sparse or limited-angle set those weights are
a poor density compensation (the two ends of a wedge get the weight of the
whole missing arc).  Here a small network proposes, for every angle and
padded spectrum position, a complex gain that multiplies the filter:

    gain[a, ky, kx] = 1 + MLP(2*kx/lNx, 2*ky/lNy, angle feature, gap feature)

(4 -> 64 -> 64 -> 64 -> 2, SiLU, BF16 tensor-core kernels
``odt_mlp_gain_forward`` / ``odt_mlp_gain_backward``).  The last layer starts
at zero, so an untrained network is the plain filter.  The network is trained
through the hand-written adjoint of the reconstruction
(``odt_bpp3d_adjoint``'s angle_gain_grad) on pairs the method itself makes:
the sparse-angle reconstruction of a random ellipsoid phantom against the
plain reconstruction of the same phantom from a dense full circle.

:class:`LearnedFilter` reconstructs with the gain and keeps the plain filter
as the fallback: it is used whenever the learned gain is disabled, e.g.
because it did not beat the plain filter on validation phantoms.
"""
import ctypes
import json
import math
import time

import numpy as np

from . import _native
from ._alg3d import Backprop3D
from . import phantoms as _ph

HIDDEN = 64
PARAM_SHAPES = {"W1": (HIDDEN, 4), "b1": (HIDDEN,), "W2": (HIDDEN, HIDDEN),
                "b2": (HIDDEN,), "W3": (HIDDEN, HIDDEN), "b3": (HIDDEN,),
                "W4": (2, HIDDEN), "b4": (2,)}


def _torch():
    import torch
    return torch


def wedge_angles(num_angles=40, span=2 * np.pi / 3, center=0.0):
    """``num_angles`` angles uniform over a wedge of ``span`` radians centred
    on ``center`` (midpoints of equal sub-intervals)."""
    step = span / num_angles
    return center - span / 2 + step * (np.arange(num_angles) + 0.5)


def angle_features(angles):
    """(A, 2) float32 per-angle features: (phi mod 2 pi)/pi - 1, and
    log(gap * A / (2 pi)) where gap is half the arc between the two
    neighbours of the angle on the circle (0 for a uniform full circle)."""
    phi = np.mod(np.asarray(angles, dtype=np.float64).ravel(), 2 * np.pi)
    A = phi.size
    order = np.argsort(phi, kind="stable")
    s = phi[order]
    if A == 1:
        gap_sorted = np.array([np.pi])
    else:
        nxt = np.roll(s, -1) - s
        nxt[-1] += 2 * np.pi
        prv = s - np.roll(s, 1)
        prv[0] += 2 * np.pi
        gap_sorted = 0.5 * (nxt + prv)
    gap = np.empty(A)
    gap[order] = gap_sorted
    gap = np.maximum(gap, 1e-6)
    out = np.empty((A, 2), dtype=np.float32)
    out[:, 0] = phi / np.pi - 1.0
    out[:, 1] = np.log(gap * A / (2 * np.pi))
    return out


class GainMLP:
    """FP32 master parameters of the gain network on one CUDA device, and
    the calls of the BF16 tensor-core kernels."""

    def __init__(self, device="cuda", seed=0):
        torch = _torch()
        device = torch.device(device)
        if device.type == "cuda" and device.index is None:
            device = torch.device("cuda", torch.cuda.current_device())
        self.device = device
        g = torch.Generator().manual_seed(int(seed))
        p = {}
        for name, shape in PARAM_SHAPES.items():
            if name == "W4" or name.startswith("b"):
                t = torch.zeros(shape)
            else:
                bound = math.sqrt(6.0 / shape[1])
                t = (torch.rand(shape, generator=g) * 2 - 1) * bound
            p[name] = t.to(self.device).requires_grad_(False)
        self.params = p
        self._packed = None
        self._packed_version = -1
        self.version = 0
        self._store = None

    # -- parameters ------------------------------------------------------
    def state(self):
        return {k: v.detach().cpu().numpy().copy()
                for k, v in self.params.items()}

    def load_state(self, state):
        torch = _torch()
        for k, shape in PARAM_SHAPES.items():
            v = np.asarray(state[k], dtype=np.float32)
            if v.shape != shape:
                raise ValueError("parameter %s has shape %s, expected %s"
                                 % (k, v.shape, shape))
            self.params[k] = torch.tensor(v, device=self.device)
        self.bump()

    def save(self, path, meta=None):
        st = self.state()
        np.savez(path, meta=json.dumps(meta or {}), **st)

    @classmethod
    def load(cls, path, device="cuda"):
        z = np.load(path, allow_pickle=False)
        m = cls(device=device)
        m.load_state({k: z[k] for k in PARAM_SHAPES})
        m.meta = json.loads(str(z["meta"])) if "meta" in z else {}
        return m

    def bump(self):
        """Mark the parameters as changed (after an optimiser step)."""
        self.version += 1

    def _pack(self):
        """BF16 device copies in the kernels' padded layouts."""
        if self._packed_version == self.version:
            return self._packed
        torch = _torch()
        bf, f32, dev = torch.bfloat16, torch.float32, self.device
        p = self.params
        w1 = torch.zeros((HIDDEN, 16), dtype=bf, device=dev)
        w1[:, :4] = p["W1"].to(bf)
        w4 = torch.zeros((8, HIDDEN), dtype=bf, device=dev)
        w4[:2] = p["W4"].to(bf)
        w4t = torch.zeros((HIDDEN, 16), dtype=bf, device=dev)
        w4t[:, :2] = p["W4"].t().to(bf)
        b4 = torch.zeros(8, dtype=f32, device=dev)
        b4[:2] = p["b4"]
        t = {
            "w1": w1, "w2": p["W2"].to(bf).contiguous(),
            "w3": p["W3"].to(bf).contiguous(), "w4": w4,
            "w2t": p["W2"].t().contiguous().to(bf),
            "w3t": p["W3"].t().contiguous().to(bf), "w4t": w4t,
            "b1": p["b1"].contiguous(), "b2": p["b2"].contiguous(),
            "b3": p["b3"].contiguous(), "b4": b4,
        }
        s = _native.MlpParams(**{k: v.data_ptr() for k, v in t.items()})
        self._packed = (t, s)
        self._packed_version = self.version
        return self._packed

    # -- kernels ---------------------------------------------------------
    def _feat(self, feat):
        torch = _torch()
        if not isinstance(feat, torch.Tensor):
            feat = torch.tensor(np.asarray(feat, dtype=np.float32))
        feat = feat.to(device=self.device, dtype=torch.float32).contiguous()
        if feat.dim() != 2 or feat.shape[1] != 2:
            raise ValueError("angle features must have shape (A, 2)")
        return feat

    def _positions(self, positions, pad_ny, pad_nx):
        """Device int32 list of flat spectrum positions (None: all)."""
        torch = _torch()
        if positions is None:
            return None, 0
        if not isinstance(positions, torch.Tensor):
            positions = torch.tensor(np.asarray(positions, dtype=np.int32))
        positions = positions.to(device=self.device,
                                 dtype=torch.int32).contiguous().reshape(-1)
        if positions.numel() < 1:
            raise ValueError("empty position list")
        return positions, int(positions.numel())

    def gains(self, feat, pad_ny, pad_nx, out=None, positions=None):
        """Complex64 gains (A, pad_ny, pad_nx) for per-angle features
        (A, 2).  With ``positions`` (flat ky*pad_nx + kx indices) only those
        entries are evaluated; the others are 1 in a new ``out`` and left
        untouched in a given one."""
        torch = _torch()
        feat = self._feat(feat)
        A = feat.shape[0]
        shape = (A, pad_ny, pad_nx)
        pos, npos = self._positions(positions, pad_ny, pad_nx)
        if out is None:
            out = (torch.empty if pos is None else torch.ones)(
                shape, dtype=torch.complex64, device=self.device)
        elif (out.dtype != torch.complex64 or tuple(out.shape) != shape
              or out.device != self.device or not out.is_contiguous()):
            raise ValueError("out must be a contiguous complex64 tensor of "
                             "shape %s on %s" % (shape, self.device))
        _t, s = self._pack()
        stream = torch.cuda.current_stream(self.device)
        L = _native.lib()
        _native.check(L.odt_mlp_gain_forward(
            ctypes.byref(s), A, pad_ny, pad_nx,
            ctypes.c_void_p(feat.data_ptr()),
            ctypes.c_void_p(pos.data_ptr() if pos is not None else 0), npos,
            ctypes.c_void_p(out.data_ptr()),
            ctypes.c_void_p(stream.cuda_stream)))
        return out

    def check(self):
        """Wait for the current stream and raise if a tensor-core wait of an
        inference gave up (odt_mlp_read_status)."""
        torch = _torch()
        stream = torch.cuda.current_stream(self.device)
        _native.check(_native.lib().odt_mlp_read_status(
            ctypes.c_void_p(stream.cuda_stream)))

    def grads(self, feat, gain_grad, positions=None):
        """Gradients of the loss with respect to the FP32 master parameters
        for the loss gradient ``gain_grad`` (complex64 (A, pad_ny, pad_nx),
        d/dRe + i d/dIm) with respect to the gains.  With ``positions`` only
        those entries contribute (exact where gain_grad is zero elsewhere,
        as it is outside the filter's support)."""
        torch = _torch()
        feat = self._feat(feat)
        A, pad_ny, pad_nx = gain_grad.shape
        if (gain_grad.dtype != torch.complex64 or not gain_grad.is_cuda
                or A != feat.shape[0]):
            raise ValueError("gain_grad must be complex64 (A, pad_ny, pad_nx)"
                             " on the device")
        gain_grad = gain_grad.contiguous()
        pos, npos = self._positions(positions, pad_ny, pad_nx)
        L = _native.lib()
        nbytes = ctypes.c_uint64()
        _native.check(L.odt_mlp_store_size(
            A, npos if pos is not None else pad_ny * pad_nx,
            ctypes.byref(nbytes)))
        if self._store is None or self._store.numel() < nbytes.value:
            self._store = torch.empty(int(nbytes.value), dtype=torch.uint8,
                                      device=self.device)
        f32, dev = torch.float32, self.device
        g = {"w1": torch.zeros((HIDDEN, 16), dtype=f32, device=dev),
             "w2": torch.zeros((HIDDEN, HIDDEN), dtype=f32, device=dev),
             "w3": torch.zeros((HIDDEN, HIDDEN), dtype=f32, device=dev),
             "w4": torch.zeros((8, HIDDEN), dtype=f32, device=dev),
             "b1": torch.zeros(HIDDEN, dtype=f32, device=dev),
             "b2": torch.zeros(HIDDEN, dtype=f32, device=dev),
             "b3": torch.zeros(HIDDEN, dtype=f32, device=dev),
             "b4": torch.zeros(8, dtype=f32, device=dev)}
        gs = _native.MlpGrads(**{k: v.data_ptr() for k, v in g.items()})
        _t, s = self._pack()
        stream = torch.cuda.current_stream(self.device)
        _native.check(L.odt_mlp_gain_backward(
            ctypes.byref(s), A, pad_ny, pad_nx,
            ctypes.c_void_p(feat.data_ptr()),
            ctypes.c_void_p(pos.data_ptr() if pos is not None else 0), npos,
            ctypes.c_void_p(gain_grad.data_ptr()),
            ctypes.c_void_p(self._store.data_ptr()), ctypes.byref(gs),
            ctypes.c_void_p(stream.cuda_stream)))
        return {"W1": g["w1"][:, :4], "b1": g["b1"], "W2": g["w2"],
                "b2": g["b2"], "W3": g["w3"], "b3": g["b3"],
                "W4": g["w4"][:2], "b4": g["b4"][:2]}


class LearnedFilter:
    """y-axis reconstruction (:class:`Backprop3D`) with the learned per-angle
    gain; the plain filter is the fallback (``enabled=False``)."""

    def __init__(self, rec, mlp, enabled=True):
        self.rec = rec
        self.mlp = mlp
        self.enabled = bool(enabled)
        self.feat = mlp._feat(angle_features(rec.angles))
        # the gain only matters where the filter is nonzero
        self.positions = mlp._positions(rec.filter_support(), 0, 0)[0]
        self._gain = None
        self._gain_version = -1

    def gains(self):
        """The gains of this angle set (computed once per parameter
        version)."""
        if self._gain_version != self.mlp.version:
            lNy, lNx = self.rec.gain_shape()
            self._gain = self.mlp.gains(self.feat, lNy, lNx, out=self._gain,
                                        positions=self.positions)
            self._gain_version = self.mlp.version
        return self._gain

    def __call__(self, sino, out=None):
        if not self.enabled:
            return self.rec(sino, out=out)
        return self.rec.forward_gain(sino, angle_gain=self.gains(), out=out)


def pretrained_path(name="wedge40_128"):
    """Path of a network shipped with the package: ``wedge40_128`` was
    trained by :func:`train_wedge_filter` with :data:`WEDGE_CONFIG` (40
    angles over a 120 degree wedge, 128^2 sinograms); its report is the
    ``.json`` beside it."""
    import os
    return os.path.join(os.path.dirname(os.path.abspath(__file__)), "data",
                        name + ".npz")


def load_learned_filter(rec, name="wedge40_128"):
    """:class:`LearnedFilter` for the plan ``rec`` with a shipped network;
    enabled as the network's validation decided (otherwise the plain
    filter)."""
    mlp = GainMLP.load(pretrained_path(name), device=rec.device)
    return LearnedFilter(rec, mlp, enabled=mlp.meta.get("enabled", True))


# ---------------------------------------------------------------------------
# Training on self-generated pairs
WEDGE_CONFIG = dict(n=128, num_angles=40, span=2 * np.pi / 3,
                    dense_angles=400, res=3.0, nm=1.333, count_range=(2, 8),
                    semi_range=(6.0, 30.0), amp_sigma=0.01, n_train=2000,
                    n_val=100, n_eval=200, epochs=4, batch=8, lr=2e-3,
                    seed=0)


def _rel_l2(a, b):
    torch = _torch()
    return (torch.linalg.vector_norm(a - b) /
            torch.linalg.vector_norm(b)).item()


def make_pairs(cfg, seeds, rec_sparse, rec_dense, sparse_angles,
               dense_angles, device):
    """Sparse sinograms and dense plain reconstructions of the phantoms
    seeded by ``seeds``: (sinos (N, A, n, n) c64, targets (N, n, n, n) c64).
    """
    torch = _torch()
    n = cfg["n"]
    N = len(seeds)
    sinos = torch.empty((N, len(sparse_angles), n, n), dtype=torch.complex64,
                        device=device)
    targets = torch.empty((N, n, n, n), dtype=torch.complex64, device=device)
    for i, sd in enumerate(seeds):
        rng = np.random.default_rng(int(sd))
        ells = _ph.random_ellipsoids(rng, n, cfg["count_range"],
                                     cfg["semi_range"])
        sp = _ph.project([ells], sparse_angles, n, cfg["res"], cfg["nm"],
                         cfg["amp_sigma"], seed=2 * int(sd), device=device)
        sinos[i] = sp[0]
        de = _ph.project([ells], dense_angles, n, cfg["res"], cfg["nm"],
                         cfg["amp_sigma"], seed=2 * int(sd) + 1,
                         device=device)
        rec_dense(de[0], out=targets[i], check=False)
    rec_dense.check()
    return sinos, targets


def evaluate(lf, sinos, targets):
    """Mean rel-L2 to the targets of the learned and the plain
    reconstructions."""
    torch = _torch()
    rec = lf.rec
    out = torch.empty(rec.volume_shape(), dtype=torch.complex64,
                      device=rec.device)
    learned, plain = [], []
    gain = lf.gains()
    for i in range(sinos.shape[0]):
        rec.forward_gain(sinos[i], angle_gain=gain, out=out, check=False)
        learned.append(_rel_l2(out, targets[i]))
        rec(sinos[i], out=out, check=False)
        plain.append(_rel_l2(out, targets[i]))
    rec.check()
    return float(np.mean(learned)), float(np.mean(plain))


def _event_ms(fn, reps):
    torch = _torch()
    for _ in range(3):
        fn()
    s, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(
        enable_timing=True)
    torch.cuda.synchronize()
    s.record()
    for _ in range(reps):
        fn()
    e.record()
    torch.cuda.synchronize()
    return s.elapsed_time(e) / reps


def train_wedge_filter(cfg=None, device="cuda", log=print):
    """Train the gain network for the wedge configuration ``cfg`` (defaults
    :data:`WEDGE_CONFIG`).  Returns (LearnedFilter, report dict)."""
    torch = _torch()
    c = dict(WEDGE_CONFIG)
    c.update(cfg or {})
    dev = torch.device(device)
    if dev.type == "cuda" and dev.index is None:
        dev = torch.device("cuda", torch.cuda.current_device())
    n, A = c["n"], c["num_angles"]
    sp_angles = wedge_angles(A, c["span"])
    de_angles = np.linspace(0, 2 * np.pi, c["dense_angles"], endpoint=False)
    rec = Backprop3D((A, n, n), sp_angles, c["res"], c["nm"],
                     input_dtype="complex64", device=dev)
    rec_dense = Backprop3D((c["dense_angles"], n, n), de_angles, c["res"],
                           c["nm"], input_dtype="complex64", device=dev)
    base = int(c["seed"]) * 10_000_000
    t0 = time.time()
    tr_s, tr_t = make_pairs(c, base + np.arange(c["n_train"]), rec, rec_dense,
                            sp_angles, de_angles, dev)
    va_s, va_t = make_pairs(c, base + 1_000_000 + np.arange(c["n_val"]), rec,
                            rec_dense, sp_angles, de_angles, dev)
    ev_s, ev_t = make_pairs(c, base + 2_000_000 + np.arange(c["n_eval"]),
                            rec, rec_dense, sp_angles, de_angles, dev)
    torch.cuda.synchronize()
    t_data = time.time() - t0
    log("pairs: %d train, %d val, %d eval in %.1f s" %
        (c["n_train"], c["n_val"], c["n_eval"], t_data))

    mlp = GainMLP(device=dev, seed=c["seed"])
    lf = LearnedFilter(rec, mlp)
    feat = lf.feat
    lNy, lNx = rec.gain_shape()
    params = [mlp.params[k] for k in PARAM_SHAPES]
    opt = torch.optim.Adam(params, lr=c["lr"])
    steps_per_epoch = c["n_train"] // c["batch"]
    total = steps_per_epoch * c["epochs"]
    sched = torch.optim.lr_scheduler.LambdaLR(
        opt, lambda s: 0.5 * (1 + math.cos(math.pi * min(s, total) / total)))
    rng = np.random.default_rng(c["seed"] + 1)
    vol = torch.empty(rec.volume_shape(), dtype=torch.complex64, device=dev)
    history = []
    t0 = time.time()
    step = 0
    for ep in range(c["epochs"]):
        perm = rng.permutation(c["n_train"])
        ep_loss = 0.0
        for b in range(steps_per_epoch):
            idx = perm[b * c["batch"]:(b + 1) * c["batch"]]
            gain = lf.gains()
            dgain = torch.zeros_like(gain)
            loss = 0.0
            for i in idx:
                rec.forward_gain(tr_s[i], angle_gain=gain, out=vol,
                                 check=False)
                tgt = tr_t[i]
                nt = torch.linalg.vector_norm(tgt) ** 2
                diff = vol - tgt
                loss += (torch.linalg.vector_norm(diff) ** 2 / nt).item()
                cot = (diff * (2.0 / (len(idx) * nt))).to(torch.complex64)
                _s, _g, ag = rec.adjoint(tr_s[i], cot, angle_gain=gain,
                                         need_sino=False,
                                         need_angle_gain=True)
                dgain += ag
            g = mlp.grads(feat, dgain, positions=lf.positions)
            for k in PARAM_SHAPES:
                mlp.params[k].grad = g[k].clone()
            opt.step()
            sched.step()
            mlp.bump()
            ep_loss += loss / len(idx)
            step += 1
        vl, vp = evaluate(lf, va_s, va_t)
        history.append({"epoch": ep, "train_loss": ep_loss / steps_per_epoch,
                        "val_rel_l2_learned": vl, "val_rel_l2_plain": vp})
        log("epoch %d: train loss %.4f, val rel-L2 learned %.4f plain %.4f"
            % (ep, ep_loss / steps_per_epoch, vl, vp))
    torch.cuda.synchronize()
    t_train = time.time() - t0
    vl, vp = evaluate(lf, va_s, va_t)
    lf.enabled = vl < vp                       # plain-filter fallback
    el, ep_ = evaluate(lf, ev_s, ev_t)
    # GPU time of one reconstruction: plain vs learned (gains cached), and
    # the gain inference itself
    sino0 = ev_s[0]
    ms_plain = _event_ms(lambda: rec(sino0, out=vol, check=False), 20)
    gain = lf.gains()
    ms_learned = _event_ms(lambda: rec.forward_gain(
        sino0, angle_gain=gain, out=vol, check=False), 20)
    ms_infer = _event_ms(lambda: mlp.gains(feat, lNy, lNx, out=gain,
                                           positions=lf.positions), 20)
    report = {
        "config": {k: (list(v) if isinstance(v, tuple) else v)
                   for k, v in c.items()},
        "eval_rel_l2_learned": el, "eval_rel_l2_plain": ep_,
        "reduction": 1.0 - el / ep_,
        "val_rel_l2_learned": vl, "val_rel_l2_plain": vp,
        "enabled": lf.enabled,
        "ms_plain": ms_plain, "ms_learned_cached_gain": ms_learned,
        "ms_gain_inference": ms_infer,
        "time_ratio_cached": ms_learned / ms_plain,
        "time_ratio_with_inference": (ms_learned + ms_infer) / ms_plain,
        "seconds_data": t_data, "seconds_train": t_train, "steps": step,
        "history": history,
    }
    log(json.dumps({k: v for k, v in report.items() if k != "history"}))
    return lf, report


if __name__ == "__main__":  # pragma: no cover - GPU training entry point
    import argparse
    ap = argparse.ArgumentParser(description=__doc__.splitlines()[0])
    ap.add_argument("--out", default=None, help="save weights (.npz)")
    ap.add_argument("--report", default=None, help="write the report (.json)")
    ap.add_argument("--n-train", type=int, default=WEDGE_CONFIG["n_train"])
    ap.add_argument("--n-val", type=int, default=WEDGE_CONFIG["n_val"])
    ap.add_argument("--n-eval", type=int, default=WEDGE_CONFIG["n_eval"])
    ap.add_argument("--epochs", type=int, default=WEDGE_CONFIG["epochs"])
    ap.add_argument("--batch", type=int, default=WEDGE_CONFIG["batch"])
    ap.add_argument("--lr", type=float, default=WEDGE_CONFIG["lr"])
    a = ap.parse_args()
    lf, rep = train_wedge_filter(dict(n_train=a.n_train, n_val=a.n_val,
                                      n_eval=a.n_eval, epochs=a.epochs,
                                      batch=a.batch, lr=a.lr))
    if a.out:
        lf.mlp.save(a.out, meta={"enabled": lf.enabled,
                                 "config": rep["config"]})
    if a.report:
        with open(a.report, "w") as f:
            json.dump(rep, f, indent=1)
