"""TEST INFRASTRUCTURE ONLY -- CPU oracle of the learned filter-gain MLP.

The learned gain has no counterpart in the reference (its filter is fixed,
odtbrain/_alg3d_bpp.py:371-399); this module is the checker of the GPU
kernels ``odt_mlp_gain_forward`` / ``odt_mlp_gain_backward``.  It restates
the network in NumPy FP64:

    x   = (2*kx/lNx, 2*ky/lNy, angle feature, gap feature)   (fftfreq order)
    z1  = W1 x + b1,   h1 = silu(z1)
    z2  = W2 h1 + b2,  h2 = silu(z2)
    z3  = W3 h2 + b3,  h3 = silu(z3)
    out = W4 h3 + b4,  gain = 1 + out[0] + i*out[1]

and its reverse mode for a real loss whose gradient with respect to the
complex gain is given in PyTorch's convention (d/dRe + i d/dIm).

``bf16=True`` rounds every tensor-core operand to BF16 (round to nearest
even) where the GPU kernels do: the weights, the features, the activations
fed to the next layer, the output gradient and the pre-activation gradients.
Sums are FP64 (the GPU accumulates in FP32).  ``bf16=False`` is the exact
FP64 network; its gradients are pinned by finite differences in the CPU
tests, which pins the reverse-mode code shared by both settings.

Only ``tests/`` may import this module.
"""
import numpy as np


def bf16_round(x):
    """Round FP32 values to the nearest BF16 (ties to even), as FP32."""
    x = np.ascontiguousarray(x, dtype=np.float32)
    u = x.view(np.uint32).astype(np.uint64)
    u = ((u + 0x7FFF + ((u >> 16) & 1)) >> 16) << 16
    return u.astype(np.uint32).view(np.float32)


def features(angle_features, lNy, lNx):
    """(A*lNy*lNx, 4) FP64 input features, point index (a*lNy + ky)*lNx + kx."""
    af = np.asarray(angle_features, dtype=np.float64).reshape(-1, 2)
    A = af.shape[0]
    # FP32 arithmetic of the kernel: 2 * float(m) / float(N), m in fftfreq
    # order
    fx = (np.float32(2.0) * np.fft.fftfreq(lNx, 1.0 / lNx).astype(np.float32)
          / np.float32(lNx)).astype(np.float64)
    fy = (np.float32(2.0) * np.fft.fftfreq(lNy, 1.0 / lNy).astype(np.float32)
          / np.float32(lNy)).astype(np.float64)
    X = np.empty((A, lNy, lNx, 4))
    X[..., 0] = fx[None, None, :]
    X[..., 1] = fy[None, :, None]
    X[..., 2] = af[:, 0, None, None].astype(np.float32)
    X[..., 3] = af[:, 1, None, None].astype(np.float32)
    return X.reshape(-1, 4)


def _silu(z):
    return z / (1.0 + np.exp(-z))


def _silu_grad(z):
    s = 1.0 / (1.0 + np.exp(-z))
    return s * (1.0 + z * (1.0 - s))


def _r(x, bf16):
    return bf16_round(x).astype(np.float64) if bf16 else np.asarray(x, float)


def forward(params, X, bf16=True):
    """params: dict W1 (64,4), b1, W2 (64,64), b2, W3, b3, W4 (2,64), b4.
    Returns (gain complex (P,), cache)."""
    W = {k: _r(params[k], bf16) for k in ("W1", "W2", "W3", "W4")}
    b = {k: np.asarray(params[k], float) for k in ("b1", "b2", "b3", "b4")}
    x = _r(X, bf16)
    z1 = x @ W["W1"].T + b["b1"]
    h1 = _r(_silu(z1), bf16)
    z2 = h1 @ W["W2"].T + b["b2"]
    h2 = _r(_silu(z2), bf16)
    z3 = h2 @ W["W3"].T + b["b3"]
    h3 = _r(_silu(z3), bf16)
    out = h3 @ W["W4"].T + b["b4"]
    gain = (1.0 + out[:, 0]) + 1j * out[:, 1]
    cache = dict(W=W, x=x, z1=z1, z2=z2, z3=z3, h1=h1, h2=h2, h3=h3)
    return gain, cache


def backward(params, X, dgain, bf16=True):
    """Gradients of the loss with respect to every parameter, given
    dgain = dL/dRe(gain) + i dL/dIm(gain) per point."""
    _, c = forward(params, X, bf16)
    W = c["W"]
    dg = np.asarray(dgain).reshape(-1)
    do = _r(np.stack([dg.real, dg.imag], axis=1), bf16)
    dz3 = _r((do @ W["W4"]) * _silu_grad(c["z3"]), bf16)
    dz2 = _r((dz3 @ W["W3"]) * _silu_grad(c["z2"]), bf16)
    dz1 = _r((dz2 @ W["W2"]) * _silu_grad(c["z1"]), bf16)
    return {
        "W4": do.T @ c["h3"], "b4": do.sum(0),
        "W3": dz3.T @ c["h2"], "b3": dz3.sum(0),
        "W2": dz2.T @ c["h1"], "b2": dz2.sum(0),
        "W1": dz1.T @ c["x"], "b1": dz1.sum(0),
    }
