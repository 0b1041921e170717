"""Dense FP64 PyTorch re-expression of the y-axis backpropagation, for
checking the hand-written adjoint with torch.autograd.

Every stage of odtbrain/_alg3d_bpp.py:285-549 is written with differentiable
torch operations at small sizes: weighting, edge padding (index clamping),
2D FFT, filter (times an optional real gain), per-plane propagator and
unnormalised inverse FFT, crop, the mirror-boundary spline prefilter as
dense matrices (built from the oracle's prefilter), and the rotation as one
dense interpolation matrix per angle (scipy.ndimage semantics: FP64
coordinates in scipy's operation order, mirror-extended taps, zero outside
[0, n-1]).  The CPU tests check this model against the oracle before the GPU
tests use it.
"""
import numpy as np
import torch

from oracle import odt_oracle as O


def _bspline(u, order):
    a = abs(u)
    if order == 1:
        return max(0.0, 1.0 - a)
    if order == 2:
        if a < 0.5:
            return 0.75 - a * a
        if a < 1.5:
            return 0.5 * (1.5 - a) ** 2
        return 0.0
    if order == 3:
        if a < 1.0:
            return 2.0 / 3.0 - a * a + 0.5 * a ** 3
        if a < 2.0:
            return (2.0 - a) ** 3 / 6.0
        return 0.0
    raise ValueError(order)


def _mirror(i, n):
    if n == 1:
        return 0
    p = 2 * n - 2
    i = abs(i) % p
    return i if i < n else p - i


def interp_matrix(mat, off, nz, nx, order):
    """(nz*nx, nz*nx) matrix mapping spline coefficients of a (z, x) plane
    to the rotated plane."""
    W = np.zeros((nz * nx, nz * nx))
    for oz in range(nz):
        for ox in range(nx):
            cz = off[0]
            cz += mat[0, 0] * oz
            cz += mat[0, 1] * ox
            cx = off[1]
            cx += mat[1, 0] * oz
            cx += mat[1, 1] * ox
            if cz < 0 or cz > nz - 1 or cx < 0 or cx > nx - 1:
                continue
            sup = (order + 1) // 2 + 1
            for tz in range(int(np.floor(cz)) - sup, int(np.floor(cz)) + sup + 1):
                wz = _bspline(cz - tz, order)
                if wz == 0.0:
                    continue
                for tx in range(int(np.floor(cx)) - sup,
                                int(np.floor(cx)) + sup + 1):
                    wx = _bspline(cx - tx, order)
                    if wx == 0.0:
                        continue
                    W[oz * nx + ox,
                      _mirror(tz, nz) * nx + _mirror(tx, nx)] += wz * wx
    return W


def prefilter_matrix(n, order):
    """Dense mirror-boundary prefilter of a length-n line (columns are the
    oracle's prefilter of unit vectors)."""
    if order < 2:
        return np.eye(n)
    return np.stack([O.spline_filter_line(np.eye(n)[i], order)
                     for i in range(n)], axis=1)


class DenseBackprop:
    """Differentiable FP64 model: __call__(sino, gain, angle_gain) -> volume
    [z,y,x]; gain (lNy, lNx) real, angle_gain (A, lNy, lNx) complex."""

    def __init__(self, angles, ny, nx, res, nm, lD=0.0, padfac=1.75,
                 order=2, weight_angles=True):
        angles = np.asarray(angles, dtype=float)
        A = angles.size
        geo = O.padding_geometry(ny, nx, (True, True), padfac)
        self.geo = geo
        self.A, self.ny, self.nx = A, ny, nx
        lNy, lNx = geo["lNy"], geo["lNx"]
        fc = O.filter_constants(A, lNx, lNy, res, nm, lD)
        pre = fc["prefactor"] * np.abs(fc["kx"]) * fc["klp"]
        pre = pre * np.exp(-1j * fc["km"] * (fc["M"] - 1) * lD)
        self.filt = torch.from_numpy(np.broadcast_to(pre / (lNx * lNy),
                                                     (lNy, lNx)).copy())
        self.phase = torch.from_numpy(np.broadcast_to(
            fc["km"] * (fc["M"] - 1), (lNy, lNx)).copy())
        nz = nx
        z = np.linspace(-nz / 2, nz / 2, nz, endpoint=False)
        self.z = torch.from_numpy(z)
        self.w = torch.from_numpy(O.compute_angle_weights_1d(angles)
                                  if weight_angles else np.ones(A))
        self.pfz = torch.from_numpy(prefilter_matrix(nz, order))
        self.pfx = torch.from_numpy(prefilter_matrix(nx, order))
        mats = []
        for phi in angles:
            m, off = O.rotate_matrix_offset((nz, nx), -np.rad2deg(phi))
            mats.append(interp_matrix(m, off, nz, nx, order))
        self.W = torch.from_numpy(np.stack(mats))  # (A, nz*nx, nz*nx)
        ys = np.clip(np.arange(lNy) - geo["padyl"], 0, ny - 1)
        xs = np.clip(np.arange(lNx) - geo["padxl"], 0, nx - 1)
        self.ys = torch.from_numpy(ys)
        self.xs = torch.from_numpy(xs)

    def __call__(self, sino, gain=None, angle_gain=None):
        g = self.geo
        lNy, lNx = g["lNy"], g["lNx"]
        s = sino * self.w.reshape(-1, 1, 1)
        padded = s[:, self.ys][:, :, self.xs]
        X = torch.fft.fft2(padded)
        F = self.filt if gain is None else self.filt * gain
        X = X * F
        if angle_gain is not None:
            X = X * angle_gain
        prop = torch.exp(1j * self.phase[None] * self.z.reshape(-1, 1, 1))
        V = X[:, None] * prop[None]                    # (A, nz, lNy, lNx)
        u = torch.fft.ifft2(V, norm="forward")
        slab = u[:, :, g["padyl"]:g["padyl"] + self.ny,
                 g["padxl"]:g["padxl"] + self.nx]      # (A, z, y, x)
        c = torch.einsum("zq,aqyx->azyx", self.pfz.to(slab.dtype), slab)
        c = torch.einsum("xk,azyk->azyx", self.pfx.to(slab.dtype), c)
        A, nz, ny, nx = c.shape
        planes = c.permute(0, 2, 1, 3).reshape(A, ny, nz * nx)  # (A, y, zx)
        out = torch.einsum("aoc,ayc->yo", self.W.to(planes.dtype), planes)
        return out.reshape(ny, nz, nx).permute(1, 0, 2)
