"""Seeded random ellipse / ellipsoid phantoms (stand-ins for the reference's
missing .mat data: trial2D, ThoraxHD_661, phantom512).

An ellipsoid adds its amplitude A to every voxel whose centre lies inside it,
as phantom3d.m:71-108 does; the sum is clipped to [0, 1].  Parameters are in
normalised coordinates (each axis of the volume spans [-1, 1]); rotation is
about the z axis by phi, as phantom3d's first Euler angle.

Draws (numpy default_rng(seed)): A ~ U[0.1, 0.5]; semi-axes ~ U[0.05, 0.45];
centres uniform in the disc (2D) / ball (3D) of radius 0.5, so every object
stays inside the inscribed circle of the field; phi ~ U[0, pi).
"""
from __future__ import annotations

import numpy as np
import torch


def ellipse_params(count: int = 10, seed: int = 0) -> np.ndarray:
    """Rows (A, a, b, x0, y0, phi), normalised units."""
    rng = np.random.default_rng(seed)
    A = rng.uniform(0.1, 0.5, count)
    ax = rng.uniform(0.05, 0.45, (count, 2))
    r = 0.5 * np.sqrt(rng.uniform(0, 1, count))
    th = rng.uniform(0, 2 * np.pi, count)
    phi = rng.uniform(0, np.pi, count)
    return np.stack([A, ax[:, 0], ax[:, 1], r * np.cos(th), r * np.sin(th), phi], axis=1)


def ellipsoid_params(count: int = 12, seed: int = 1) -> np.ndarray:
    """Rows (A, a, b, c, x0, y0, z0, phi), normalised units."""
    rng = np.random.default_rng(seed)
    A = rng.uniform(0.1, 0.5, count)
    ax = rng.uniform(0.05, 0.45, (count, 3))
    v = rng.normal(size=(count, 3))
    v /= np.linalg.norm(v, axis=1, keepdims=True)
    r = 0.5 * rng.uniform(0, 1, count) ** (1.0 / 3.0)
    c = v * r[:, None]
    phi = rng.uniform(0, np.pi, count)
    return np.stack([A, ax[:, 0], ax[:, 1], ax[:, 2], c[:, 0], c[:, 1], c[:, 2], phi], axis=1)


def _axis(n, device):
    return (torch.arange(n, device=device, dtype=torch.float64) + 0.5) * (2.0 / n) - 1.0


def ellipses_2d(n_t: int, n_s: int, params: np.ndarray, device="cpu") -> torch.Tensor:
    """float32 image [s][t]."""
    u = _axis(n_t, device)[None, :]
    v = _axis(n_s, device)[:, None]
    img = torch.zeros(n_s, n_t, dtype=torch.float64, device=device)
    for A, a, b, x0, y0, phi in params:
        c, s = np.cos(phi), np.sin(phi)
        xr = (u - x0) * c + (v - y0) * s
        yr = -(u - x0) * s + (v - y0) * c
        img += A * ((xr / a) ** 2 + (yr / b) ** 2 <= 1.0)
    return img.clamp_(0.0, 1.0).to(torch.float32)


def ellipsoids_3d(n_t: int, n_s: int, n_z: int, params: np.ndarray, device="cpu") -> torch.Tensor:
    """float32 volume [z][s][t], built slab by slab to bound temporary memory."""
    vol = torch.zeros(n_z, n_s, n_t, dtype=torch.float32, device=device)
    u = _axis(n_t, device).to(torch.float32)[None, None, :]
    v = _axis(n_s, device).to(torch.float32)[None, :, None]
    w_all = _axis(n_z, device).to(torch.float32)
    slab = max(1, min(n_z, (1 << 26) // max(1, n_t * n_s)))
    for z0 in range(0, n_z, slab):
        w = w_all[z0:z0 + slab][:, None, None]
        acc = torch.zeros(w.shape[0], n_s, n_t, dtype=torch.float32, device=device)
        for A, a, b, c_, x0, y0, zz, phi in params:
            c, s = float(np.cos(phi)), float(np.sin(phi))
            xr = (u - x0) * c + (v - y0) * s
            yr = -(u - x0) * s + (v - y0) * c
            zr = w - zz
            acc += float(A) * ((xr / a) ** 2 + (yr / b) ** 2 + (zr / c_) ** 2 <= 1.0)
        vol[z0:z0 + slab] = acc.clamp_(0.0, 1.0)
    return vol


def phantom3d(n: int, ellipsoids, device="cpu") -> torch.Tensor:
    """The voxel rule of phantom3d.m:71-108 on its own n^3 grid, returned in the
    layout the reference's 3D scripts hand to the operators.

    * Grid: voxel centres at ((0:n-1) - (n-1)/2) / ((n-1)/2), the end points
      -1 and 1 included (phantom3d.m:73), not the cell centres of ellipsoids_3d.
    * Rows (A, a, b, c, x0, y0, z0, phi) with phi in degrees about z
      (phantom3d.m:87); a voxel gets the sum of the amplitudes of every
      ellipsoid containing its centre, ((R (p - p0)) / (a, b, c))^2 summed <= 1,
      R the rotation by phi; no clipping.
    * Layout: meshgrid puts x along MATLAB's second index and y along the first,
      and SIRT3D.m:51-57 vectorises pic(t, s, z) with t fastest, so the result is
      float32 [z][s][t] with x along s and y along t."""
    r = (torch.arange(n, device=device, dtype=torch.float64) - (n - 1) / 2.0) / ((n - 1) / 2.0)
    y = r[None, None, :]          # t index
    x = r[None, :, None]          # s index
    z = r[:, None, None]          # z index
    vol = torch.zeros(n, n, n, dtype=torch.float64, device=device)
    for A, a, b, c_, x0, y0, z0, phi in ellipsoids:
        ph = float(phi) * np.pi / 180.0
        cp, sp = float(np.cos(ph)), float(np.sin(ph))
        xr = cp * (x - x0) + sp * (y - y0)
        yr = -sp * (x - x0) + cp * (y - y0)
        vol += float(A) * ((xr / a) ** 2 + (yr / b) ** 2 + ((z - z0) / c_) ** 2 <= 1.0)
    return vol.to(torch.float32)


def world_ellipsoids(params: np.ndarray, size) -> list:
    """Normalised ellipsoid rows -> world-frame rows (A, a, b, c, x0, y0, z0, phi)
    in mm for a volume spanning [0, Size]; requires Size_t == Size_s so the
    rotation about z stays a rotation."""
    St, Ss, Sz = size
    if abs(St - Ss) > 1e-9 * St:
        raise ValueError("world_ellipsoids needs Size_t == Size_s")
    h, hz = St / 2.0, Sz / 2.0
    return [(A, a * h, b * h, c * hz, St / 2 + x0 * h, Ss / 2 + y0 * h, Sz / 2 + z0 * hz, phi)
            for A, a, b, c, x0, y0, z0, phi in params]


def poisson_noise(sino: torch.Tensor, photons: float = 1e5, max_integral: float = 4.0, seed: int = 3):
    """Scale line integrals so the largest is `max_integral`, draw
    I ~ Poisson(photons * exp(-p)) and return (-ln(max(I,1)/photons) / scale, scale)."""
    scale = max_integral / float(sino.max().clamp_min(1e-12))
    g = torch.Generator(device=sino.device)
    g.manual_seed(seed)
    lam = photons * torch.exp(-sino.double() * scale)
    counts = torch.poisson(lam, generator=g).clamp_min_(1.0)
    return (-torch.log(counts / photons) / scale).to(torch.float32), scale
