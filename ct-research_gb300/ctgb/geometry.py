"""Scan geometries in the reference's parameterisation, and the benchmark workloads.

The reference describes a cone scan by the volume size (t, s, z), its extent
Size (mm), the source-to-centre distance D, the view angles BetaScanRange
(radians) and the coordinates of a virtual flat detector through the rotation
centre, Pdomain (in-plane) and Xigamadomain (axial) (FDK_GPU.m:33-68,
ProjectionCone_3D.cpp:5-22).  A physical detector at source-detector distance
SDD with pitch p maps onto that virtual detector with pitch p * D / SDD.
Angles follow SIRT.m:17-19: beta_k = k * 2pi / n_views, k = 1..n_views.
"""
from __future__ import annotations

from dataclasses import dataclass, field

import numpy as np


def view_angles(n_views: int, arc: float = 2 * np.pi) -> np.ndarray:
    """BetaScanInt : BetaScanInt : MaxBeta with BetaScanInt = arc / n_views."""
    return (np.arange(1, n_views + 1, dtype=np.float64) * (arc / n_views))


def centred_domain(n: int, pitch: float) -> np.ndarray:
    """n detector coordinates (i - (n-1)/2) * pitch, i = 0..n-1."""
    return (np.arange(n, dtype=np.float64) - (n - 1) / 2.0) * pitch


@dataclass
class ConeGeometry:
    """Circular cone-beam scan (ProjectionCone_3D / Backprojection3D / FDK)."""
    nt: int
    ns: int
    nz: int
    size: tuple            # (Size_t, Size_s, Size_z) in mm
    beta: np.ndarray       # float32 radians
    P: np.ndarray          # float32 mm, virtual detector columns
    xi: np.ndarray         # float32 mm, virtual detector rows
    D: float               # source to rotation centre, mm
    name: str = ""

    def __post_init__(self):
        self.beta = np.ascontiguousarray(self.beta, np.float32)
        self.P = np.ascontiguousarray(self.P, np.float32)
        self.xi = np.ascontiguousarray(self.xi, np.float32)
        self.size = tuple(float(s) for s in self.size)

    @property
    def vol_shape(self):
        return (self.nz, self.ns, self.nt)

    @property
    def sino_shape(self):
        return (len(self.beta), len(self.xi), len(self.P))

    @property
    def n_rays(self) -> int:
        return len(self.beta) * len(self.xi) * len(self.P)

    @property
    def n_voxels(self) -> int:
        return self.nt * self.ns * self.nz

    def with_views(self, n_views: int) -> "ConeGeometry":
        return ConeGeometry(self.nt, self.ns, self.nz, self.size, view_angles(n_views), self.P, self.xi,
                            self.D, self.name)

    def subset_views(self, idx) -> "ConeGeometry":
        return ConeGeometry(self.nt, self.ns, self.nz, self.size, self.beta[idx], self.P, self.xi, self.D,
                            self.name)


@dataclass
class FanGeometry:
    """2D fan-beam scan (ProjectionFan_2D / BackprojectionFan2D / FBPfan)."""
    nt: int
    ns: int
    size: tuple            # (Size_t, Size_s) mm
    beta: np.ndarray       # float64 radians (ProjectionFan_2D takes doubles)
    P: np.ndarray          # float64 mm
    D: float               # Rscan
    name: str = ""

    def __post_init__(self):
        self.beta = np.ascontiguousarray(self.beta, np.float64)
        self.P = np.ascontiguousarray(self.P, np.float64)
        self.size = tuple(float(s) for s in self.size)

    @property
    def img_shape(self):
        return (self.ns, self.nt)

    @property
    def sino_shape(self):
        return (len(self.beta), len(self.P))


def cone_from_physical(n_vox, size, n_views, det_cols, det_rows, pitch, sid, sdd, name="") -> ConeGeometry:
    """Map a physical flat detector (pitch at distance sdd) onto the reference's
    virtual detector through the centre (pitch * sid / sdd)."""
    iso = pitch * sid / sdd
    nt, ns, nz = n_vox
    return ConeGeometry(nt, ns, nz, size, view_angles(n_views), centred_domain(det_cols, iso),
                        centred_domain(det_rows, iso), sid, name)


def fan_config(n: int = 256, n_views: int = 360, n_det: int = 512, D: float = 500.0, size: float | None = None,
               name: str = "fan2d") -> FanGeometry:
    """2D fan scan with the reference's detector convention (SIRT.m:25-39):
    MaxP = 1.1 * Size * sqrt(2)/2, n_det bins spanning [-MaxP, MaxP]."""
    size = float(n) if size is None else float(size)
    maxp = 1.1 * size * np.sqrt(2.0) / 2.0
    P = np.linspace(-maxp, maxp, n_det)
    return FanGeometry(n, n, (size, size), view_angles(n_views), P, D, name)


# -- the benchmark workloads ---------------------------------------------------

def config_fan2d() -> FanGeometry:
    """2D fan FP + FBP: 256^2, 360 views over 360 deg, 512 bins, source-iso 500 mm,
    source-detector 1000 mm (rescales the physical pitch only)."""
    return fan_config(256, 360, 512, 500.0, 256.0, name="fan2d_256")


def config_cone_fdk() -> ConeGeometry:
    """3D cone FDK: 256^3 over 128 mm, 360 views, 512x384 detector at 0.8 mm,
    SID 600 / SDD 1200 (0.4 mm at the centre)."""
    return cone_from_physical((256, 256, 256), (128.0, 128.0, 128.0), 360, 512, 384, 0.8, 600.0, 1200.0,
                              name="cone_fdk_256")


def config_cone_512() -> ConeGeometry:
    """SIRT3D + TV workload: 512^3 over 200x200x150 mm, 360 views, 768x512
    detector at 0.8 mm, SID 600 / SDD 1200.  One forward + back projection of it
    is the throughput workload."""
    return cone_from_physical((512, 512, 512), (200.0, 200.0, 150.0), 360, 768, 512, 0.8, 600.0, 1200.0,
                              name="cone_512")


def config_batched_fan(n_slices: int = 64, seed: int = 4):
    """Batched uneven 2D fan SIRT: per slice N ~ U{128..512}, views ~ U{90..720},
    detector bins ~ U{256..1024}; Size = N mm, D = 500 mm."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(n_slices):
        n = int(rng.integers(128, 513))
        nv = int(rng.integers(90, 721))
        nd = int(rng.integers(256, 1025))
        out.append(fan_config(n, nv, nd, 500.0, float(n), name=f"slice{i}"))
    return out


def iterative_fdk_setup(size, shape, pint: float = 0.4, D: float = 200.0, n_views: int = 360):
    """Domains of the IterativeFDK error computation, as IterativeFDK.m sets
    them up (:20-60 and :294-312): returns (beta float32, U float32, P float64,
    G float64).

    * P: -MaxP .. MaxP in steps of pint, MaxP = 1.1 * max(Size) * sqrt(2)/2;
    * beta: n_views angles k * 2pi/n_views, k = 1..n_views;
    * U: LU = floor(2 Rpic / dU) depths Rpic - dU * (1..LU) along the ray,
      Rpic = max(Size) * sqrt(3)/2 and dU = max(Size) / t_length;
    * G: the Shepp-Logan taps of pint in double, 2 LP - 1 of them.
    """
    size = [float(x) for x in size]
    nz, ns, nt = shape
    ms = max(size)
    maxp = 1.1 * ms * np.sqrt(2.0) / 2.0
    n_p = int(np.floor(2 * maxp / pint + 1e-9)) + 1
    P = -maxp + pint * np.arange(n_p, dtype=np.float64)
    beta = (np.arange(1, n_views + 1) * (2 * np.pi / n_views)).astype(np.float32)
    rpic = ms * np.sqrt(3.0) / 2.0
    du = ms / nt
    lu = int(np.floor(2 * rpic / du))
    U = (rpic - du * np.arange(1, lu + 1)).astype(np.float32)
    n = np.arange(1, n_p, dtype=np.float64)
    G = np.zeros(2 * n_p - 1)
    G[n_p - 1] = 1.0 / (np.pi * pint) ** 2
    G[n_p - 1 + n.astype(int)] = G[n_p - 1 - n.astype(int)] = -1.0 / (np.pi * pint) ** 2 / (4 * n ** 2 - 1)
    return beta, U, P, G


def curved_fdk_case(kind: str = "filter"):
    """Inputs of the curved-detector FDK cases (the scanner set-up of
    ImplementUIData.m:7-36 and small variants).  Returns a dict with gama
    (descending, as the script negates the detector angles), xi, beta, b0,
    maxg (the fan angle |gama_end - gama_1|), D, ds2d and, for "bp", the
    display Size and z_length.

    * "filter": the reference's fixed detector (936 gammas at 9.7527e-4 rad,
      80 rows at 0.915 mm), D 570, SDD 1060.2, five views chosen across the
      three Parker regions.
    * "bp": a small detector (120 x 16) and a 40 x 36 x 10 display, D 100.
    * "scanner": the script's full set-up, 800 views over 240 deg from 1.5466 deg
      and a 512 x 512 x 50 display over 23 mm.
    """
    if kind in ("filter", "scanner"):
        gint = 9.7527e-4
        gama = -(np.arange(936) - 467.5) * gint
        xi = (np.arange(80) - 39.5) * 0.915
        b0 = np.deg2rad(1.5466)
        d = dict(gama=gama, xi=xi, b0=b0, maxg=abs(gama[-1] - gama[0]), D=570.0, ds2d=1060.2)
        if kind == "filter":
            d["beta"] = b0 + np.array([0.0, 0.3, 1.4, np.pi - 0.2, np.pi + 0.55])
        else:
            bint = np.deg2rad(240 / 800)
            d["beta"] = b0 + bint * np.arange(800)
            d["size"], d["z_length"] = np.array([512, 512, 23], np.int32), 50
        return d
    if kind == "bp":
        gama = -(np.arange(120) - 59.5) * 0.0075
        xi = (np.arange(16) - 7.5) * 2.2
        b0 = 0.05
        beta = b0 + np.arange(90) * (2 * np.pi / 90)
        return dict(gama=gama, xi=xi, beta=beta, b0=b0, maxg=abs(gama[-1] - gama[0]), D=100.0, ds2d=180.0,
                    size=np.array([40, 36, 13], np.int32), z_length=10)
    raise ValueError(kind)

