"""Seeded ellipsoid phantoms and their Rytov sinograms, on the GPU.

The learned filter gain is trained on pairs the method generates itself:
random ellipsoid phantoms, projected analytically for each rotation angle
about the y axis, reconstructed from a sparse angle set (the input) and from
a dense one (the target).  This module makes the sinograms:

* :func:`random_ellipsoids` draws, from a NumPy generator, 1..K ellipsoids
  inside the volume's inscribed sphere: centre, semi-axes, orientation (unit
  quaternion) and refractive index;
* :func:`project` evaluates, with PyTorch on the device, the chord length of
  every detector ray through every ellipsoid for every angle and forms the
  Rytov data  a + i*(2*pi/res) * sum (n - nm) * chord,  a ~ N(0, amp_sigma).

Geometry: detector pixel (y, x) looks along +z through the phantom rotated by
angle phi about y, pixel centres at index - (n-1)/2.
"""
import numpy as np


def _torch():
    import torch
    return torch


def random_ellipsoids(rng, n, count_range, semi_range,
                      dn_range=(1.335, 1.36)):
    """List of (centre (3,), semi-axes (3,), rotation (3, 3), index) in
    voxel units relative to the volume centre, x/y/z order."""
    count = int(rng.integers(count_range[0], count_range[1] + 1))
    out = []
    for _ in range(count):
        s = rng.uniform(semi_range[0], semi_range[1], 3)
        rmax = max(0.0, n / 2 - 1 - s.max())
        while True:
            c = rng.uniform(-rmax, rmax, 3)
            if np.linalg.norm(c) <= rmax:
                break
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([
            [1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
            [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
            [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)],
        ])
        out.append((c, s, R, rng.uniform(dn_range[0], dn_range[1])))
    return out


def _rot_y(phi):
    """Rotation matrices about y, (A, 3, 3): x' = cos x + sin z,
    z' = -sin x + cos z."""
    c, s = np.cos(phi), np.sin(phi)
    R = np.zeros((len(phi), 3, 3))
    R[:, 0, 0] = c
    R[:, 0, 2] = s
    R[:, 1, 1] = 1.0
    R[:, 2, 0] = -s
    R[:, 2, 2] = c
    return R


def project(phantoms, angles, n, res=3.0, nm=1.333, amp_sigma=0.0,
            seed=None, device="cuda", ny=None):
    """Rytov sinograms of a batch of phantoms.

    phantoms: list (length B) of lists from :func:`random_ellipsoids`.
    Returns a complex64 tensor (B, A, ny, n) on ``device``.  The noise
    a ~ N(0, amp_sigma) comes from a torch generator seeded with ``seed``.
    """
    torch = _torch()
    ny = n if ny is None else ny
    angles = np.asarray(angles, dtype=np.float64)
    A, B = angles.size, len(phantoms)
    K = max(1, max(len(p) for p in phantoms))
    # per (phantom, ellipsoid, angle): quadratic form Q and rotated centre,
    # in FP64 on the host (small), padded ellipsoids carry dn = 0
    Rphi = _rot_y(angles)
    Q = np.zeros((B, K, A, 3, 3))
    cr = np.zeros((B, K, A, 3))
    dn = np.zeros((B, K))
    for b, ells in enumerate(phantoms):
        for k, (c, s, R, nidx) in enumerate(ells):
            Rr = Rphi @ R
            Q[b, k] = Rr @ np.diag(1.0 / np.asarray(s) ** 2) @ \
                np.transpose(Rr, (0, 2, 1))
            cr[b, k] = Rphi @ np.asarray(c)
            dn[b, k] = nidx - nm
    f32 = torch.float32
    Qd = torch.tensor(Q, dtype=f32, device=device)
    crd = torch.tensor(cr, dtype=f32, device=device)
    dnd = torch.tensor(dn, dtype=f32, device=device)
    xs = torch.arange(n, dtype=f32, device=device) - (n - 1) / 2
    ys = torch.arange(ny, dtype=f32, device=device) - (ny - 1) / 2
    path = torch.zeros((B, A, ny, n), dtype=f32, device=device)
    for k in range(K):
        q = Qd[:, k][:, :, None, None]            # (B, A, 1, 1, 3, 3)
        dx = xs[None, None, None, :] - crd[:, k, :, 0][:, :, None, None]
        dy = ys[None, None, :, None] - crd[:, k, :, 1][:, :, None, None]
        qa = q[..., 2, 2]
        qb = 2 * (dx * q[..., 0, 2] + dy * q[..., 1, 2])
        qc = (q[..., 0, 0] * dx * dx + 2 * q[..., 0, 1] * dx * dy
              + q[..., 1, 1] * dy * dy - 1)
        disc = qb * qb - 4 * qa * qc
        chord = torch.sqrt(torch.clamp(disc, min=0)) / qa
        path += chord * dnd[:, k][:, None, None, None]
    phase = (2 * np.pi / res) * path
    if amp_sigma > 0:
        g = torch.Generator(device=device)
        g.manual_seed(int(seed) if seed is not None else 0)
        amp = torch.randn((B, A, ny, n), generator=g, device=device,
                          dtype=f32) * amp_sigma
    else:
        amp = torch.zeros_like(phase)
    return torch.complex(amp, phase)
