"""Device-resident operators on torch CUDA tensors (plans over libctgb).

A plan uploads the scan geometry once; its methods take and return float32
CUDA tensors in the reference layouts and queue work on the current torch
stream.  This is the path the SIRT loops use: data never leaves HBM.
"""
from __future__ import annotations

import ctypes as C

import numpy as np
import torch

from . import _lib
from .geometry import ConeGeometry, FanGeometry

FDK_FILTER_CLEAN, FDK_FILTER_LAUNCH_ORDER = 0, 1
FDK_BP_ZERO, FDK_BP_STICKY = 0, 1
FILTERS = {"shepp-logan": 0, "ram-lak": 1}


def filter_kind(kind) -> int:
    """CT_FILTER_* value of a filter name ("shepp-logan", "ram-lak") or int."""
    if isinstance(kind, str):
        if kind.lower() not in FILTERS:
            raise ValueError(f"unknown filter {kind!r}; expected one of {sorted(FILTERS)}")
        return FILTERS[kind.lower()]
    return int(kind)


def _np_ptr(a):
    return a.ctypes.data_as(C.c_void_p)


def _tptr(t: torch.Tensor):
    if t is None:
        return None
    if not t.is_cuda:
        raise ValueError("expected a CUDA tensor")
    if t.dtype not in (torch.float32, torch.float64):
        raise ValueError("expected float32 (or float64 scratch) tensor")
    if not t.is_contiguous():
        raise ValueError("expected a contiguous tensor")
    return C.c_void_p(t.data_ptr())


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def set_graze_list_capacity(cap: int) -> None:
    """List capacity of grazing-ray buffers allocated from now on (process-wide;
    the results do not depend on it: rays past the list take the overflow map)."""
    _lib.call("ct_set_graze_list_capacity", int(cap))


def _grazing(fn, h) -> int:
    n = C.c_longlong()
    _lib.call(fn, h, C.byref(n), _stream())
    return int(n.value)


class CsrMatrix:
    """A projector's system matrix in CSR on the device: row_ptr int64 (rows + 1),
    col int32, val float32 (segment lengths in mm)."""

    def __init__(self, row_ptr: torch.Tensor, col: torch.Tensor, val: torch.Tensor, shape):
        self.row_ptr, self.col, self.val, self.shape = row_ptr, col, val, tuple(shape)

    @property
    def nnz(self) -> int:
        return int(self.val.numel())

    def to_torch(self) -> torch.Tensor:
        """torch sparse CSR tensor (int64 indices) on the same device."""
        import warnings
        with warnings.catch_warnings():
            warnings.simplefilter("ignore", UserWarning)     # torch marks sparse CSR as beta
            return torch.sparse_csr_tensor(self.row_ptr, self.col.long(), self.val, size=self.shape)

    def to_scipy(self):
        from scipy.sparse import csr_matrix
        return csr_matrix((self.val.cpu().numpy(), self.col.cpu().numpy(), self.row_ptr.cpu().numpy()),
                          shape=self.shape)

    def matvec(self, x: torch.Tensor) -> torch.Tensor:
        return torch.mv(self.to_torch(), x.reshape(-1))


def _export(fn, rows: int, cols: int, device, *head) -> CsrMatrix:
    """Two-call CSR export of ct_*_sysmat: sizes, then entries."""
    row_ptr = torch.empty(rows + 1, dtype=torch.int64, device=device)
    nnz = C.c_longlong()
    _lib.call(fn, *head, C.c_void_p(row_ptr.data_ptr()), None, None, 0, C.byref(nnz), _stream())
    n = int(nnz.value)
    col = torch.empty(max(n, 1), dtype=torch.int32, device=device)
    val = torch.empty(max(n, 1), dtype=torch.float32, device=device)
    _lib.call(fn, *head, C.c_void_p(row_ptr.data_ptr()), C.c_void_p(col.data_ptr()), C.c_void_p(val.data_ptr()),
              n, C.byref(nnz), _stream())
    return CsrMatrix(row_ptr, col[:n], val[:n], (rows, cols))


class ConePlan:
    """Cone-beam operators for one ConeGeometry (ct_cone_plan_*)."""

    def __init__(self, geom: ConeGeometry, fdk_filter: int = FDK_FILTER_LAUNCH_ORDER, fdk_bp: int = FDK_BP_STICKY):
        self.geom = geom
        self._h = C.c_void_p()
        size = np.asarray(geom.size, np.float64)
        self._keep = (size, geom.beta, geom.P, geom.xi)
        _lib.call("ct_cone_plan_create", C.byref(self._h), geom.nt, geom.ns, geom.nz, _np_ptr(size),
                  _np_ptr(geom.beta), len(geom.beta), _np_ptr(geom.P), len(geom.P), _np_ptr(geom.xi),
                  len(geom.xi), float(geom.D))
        _lib.call("ct_cone_plan_set_fdk_mode", self._h, int(fdk_filter), int(fdk_bp))
        self._norms = None
        self.bp_chunk = 0

    def set_bp_chunk(self, views: int):
        """Views per backprojection chunk (0: automatic, the default; >= the
        view count: one pass)."""
        _lib.call("ct_cone_plan_set_bp_chunk", self._h, int(views))
        self.bp_chunk = int(views)
        return self

    def bp_chunk_views(self) -> int:
        """Views per backprojection chunk in effect."""
        n = C.c_int()
        _lib.call("ct_cone_plan_get_bp_chunk", self._h, C.byref(n))
        return int(n.value)

    def launches_per_pair(self) -> int:
        """Kernels of one fp + bp: layout transpose, walk, grazing re-walk, and
        per backprojection chunk the quad packing and the backprojection."""
        nb = len(self.geom.beta)
        return 3 + 2 * -(-nb // self.bp_chunk_views())

    def set_filter(self, kind="shepp-logan", window: int = 0, short_scan: bool = False):
        """FDK filter stage: ramp taps, Hamming smoothing window length (0 =
        none) and short-scan (Parker) weights.  The defaults are the reference's."""
        _lib.call("ct_cone_plan_set_filter", self._h, filter_kind(kind), int(window))
        _lib.call("ct_cone_plan_set_short_scan", self._h, int(bool(short_scan)))
        return self

    def close(self):
        if self._h:
            _lib.lib().ct_cone_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def new_volume(self, device="cuda"):
        return torch.zeros(self.geom.vol_shape, dtype=torch.float32, device=device)

    def new_sino(self, device="cuda"):
        return torch.zeros(self.geom.sino_shape, dtype=torch.float32, device=device)

    def fp(self, vol: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        out = self.new_sino(vol.device) if out is None else out
        _lib.call("ct_cone_fp", self._h, _tptr(vol), _tptr(out), _stream())
        return out

    def fp_residual(self, vol, b, rowsum=None, eps=0.0, out=None, norms=None):
        """out = (b - A vol) / (rowsum + eps); norms (float64[2]) += (|b - A vol|^2, |b|^2)."""
        out = torch.empty_like(b) if out is None else out
        if norms is None:
            norms = torch.zeros(2, dtype=torch.float64, device=vol.device)
        _lib.call("ct_cone_fp_residual", self._h, _tptr(vol), _tptr(b), _tptr(rowsum), float(eps), _tptr(out),
                  _tptr(norms), _stream())
        return out, norms

    def bp(self, proj: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        out = self.new_volume(proj.device) if out is None else out
        _lib.call("ct_cone_bp", self._h, _tptr(proj), _tptr(out), _stream())
        return out

    def bp_update(self, proj, colsum, vol, lam=1.0, eps=0.0, lo=0.0, hi=float("inf")):
        """vol = clamp(vol + lam * BP(proj) / (colsum + eps), lo, hi), in place."""
        _lib.call("ct_cone_bp_update", self._h, _tptr(proj), _tptr(colsum), float(eps), float(lam), float(lo),
                  float(hi), _tptr(vol), _stream())
        return vol

    def fdk(self, proj: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        out = self.new_volume(proj.device) if out is None else out
        _lib.call("ct_cone_fdk", self._h, _tptr(proj), _tptr(out), _stream())
        return out

    def fdk_filter(self, proj: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """Cosine pre-weight + S-L ramp of every detector row (FDK's first stage)."""
        out = torch.empty_like(proj) if out is None else out
        _lib.call("ct_cone_fdk_filter", self._h, _tptr(proj), _tptr(out), _stream())
        return out

    def fdk_bp(self, filtered: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
        """LR^2-weighted backprojection of a filtered sinogram (FDK's second stage)."""
        out = self.new_volume(filtered.device) if out is None else out
        _lib.call("ct_cone_fdk_bp", self._h, _tptr(filtered), _tptr(out), _stream())
        return out

    def sysmat(self, view0: int = 0, nviews: int | None = None, device="cuda") -> CsrMatrix:
        """CSR system matrix of views view0 .. view0 + nviews - 1 (ct_cone_sysmat):
        A vol equals fp(vol) on those views to float rounding."""
        g = self.geom
        nviews = len(g.beta) - view0 if nviews is None else int(nviews)
        rows = nviews * len(g.xi) * len(g.P)
        return _export("ct_cone_sysmat", rows, g.nt * g.ns * g.nz, device, self._h, int(view0), nviews)

    def count_segments(self) -> int:
        n = C.c_longlong()
        _lib.call("ct_cone_count_segments", self._h, C.byref(n), _stream())
        return int(n.value)

    def grazing_rays(self) -> int:
        """Rays of the last forward projection that took the FP64 re-walk."""
        return _grazing("ct_cone_plan_grazing_rays", self._h)

    def workspace_bytes(self) -> int:
        return int(_lib.lib().ct_cone_plan_workspace_bytes(self._h))


class FanPlan:
    """2D fan-beam operators for one FanGeometry (ct_fan_plan_*)."""

    def __init__(self, geom: FanGeometry):
        self.geom = geom
        self._h = C.c_void_p()
        size = np.asarray(geom.size, np.float64)
        self._keep = (size, geom.beta, geom.P)
        _lib.call("ct_fan_plan_create", C.byref(self._h), geom.nt, geom.ns, _np_ptr(size), _np_ptr(geom.beta),
                  len(geom.beta), _np_ptr(geom.P), len(geom.P), float(geom.D))

    def set_filter(self, kind="shepp-logan", window: int = 0, short_scan: bool = False):
        """FBP filter stage options, as ConePlan.set_filter."""
        _lib.call("ct_fan_plan_set_filter", self._h, filter_kind(kind), int(window))
        _lib.call("ct_fan_plan_set_short_scan", self._h, int(bool(short_scan)))
        return self

    def close(self):
        if self._h:
            _lib.lib().ct_fan_plan_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def new_image(self, device="cuda"):
        return torch.zeros(self.geom.img_shape, dtype=torch.float32, device=device)

    def sysmat(self, device="cuda") -> CsrMatrix:
        """CSR system matrix (ct_fan_sysmat): rows [beta][P], columns s * t_length + t."""
        g = self.geom
        return _export("ct_fan_sysmat", len(g.beta) * len(g.P), g.nt * g.ns, device, self._h)

    def new_sino(self, device="cuda"):
        return torch.zeros(self.geom.sino_shape, dtype=torch.float32, device=device)

    def fp(self, img, out=None):
        out = self.new_sino(img.device) if out is None else out
        _lib.call("ct_fan_fp", self._h, _tptr(img), _tptr(out), _stream())
        return out

    def fp_residual(self, img, b, rowsum=None, eps=0.0, out=None, norms=None):
        out = torch.empty_like(b) if out is None else out
        if norms is None:
            norms = torch.zeros(2, dtype=torch.float64, device=img.device)
        _lib.call("ct_fan_fp_residual", self._h, _tptr(img), _tptr(b), _tptr(rowsum), float(eps), _tptr(out),
                  _tptr(norms), _stream())
        return out, norms

    def bp(self, proj, out=None):
        out = self.new_image(proj.device) if out is None else out
        _lib.call("ct_fan_bp", self._h, _tptr(proj), _tptr(out), _stream())
        return out

    def bp_update(self, proj, colsum, img, lam=1.0, eps=0.0, lo=0.0, hi=float("inf")):
        _lib.call("ct_fan_bp_update", self._h, _tptr(proj), _tptr(colsum), float(eps), float(lam), float(lo),
                  float(hi), _tptr(img), _stream())
        return img

    def fbp(self, proj, out=None, filter_mode=FDK_FILTER_LAUNCH_ORDER):
        out = self.new_image(proj.device) if out is None else out
        _lib.call("ct_fan_fbp", self._h, _tptr(proj), _tptr(out), int(filter_mode), _stream())
        return out

    def grazing_rays(self) -> int:
        """Rays of the last forward projection that took the FP64 re-walk."""
        return _grazing("ct_fan_plan_grazing_rays", self._h)


class ParPlan(FanPlan):
    """2D parallel-beam operators (ct_par_plan_create: the ProjectionParallel_2D
    geometry, image height x width, resolution = (along height, along width))."""

    def __init__(self, height: int, width: int, resolution, theta, t_range):
        res = np.ascontiguousarray(resolution, np.float64)
        theta = np.ascontiguousarray(theta, np.float64)
        t_range = np.ascontiguousarray(t_range, np.float64)
        self.geom = FanGeometry(int(width), int(height), (res[1] * width, res[0] * height), theta, t_range, 0.0,
                                "parallel")
        self._h = C.c_void_p()
        self._keep = (res, theta, t_range)
        _lib.call("ct_par_plan_create", C.byref(self._h), int(height), int(width), _np_ptr(res), _np_ptr(theta),
                  len(theta), _np_ptr(t_range), len(t_range))


def iterfdk_err(pic: torch.Tensor, beta, U, P, G, size, D: float, t: int, out: torch.Tensor | None = None):
    """IterativeFDK error slice of image slice t (0-based) of the CUDA volume
    pic [z][s][t]: returns [beta][z][s] float32 on the device (ct_iterfdk_err)."""
    nz, ns, nt = pic.shape
    beta = np.ascontiguousarray(beta, np.float32)
    U = np.ascontiguousarray(U, np.float32)
    P = np.ascontiguousarray(P, np.float64)
    G = np.ascontiguousarray(G, np.float64)
    size = np.ascontiguousarray(size, np.float64)
    if out is None:
        out = torch.empty((len(beta), nz, ns), dtype=torch.float32, device=pic.device)
    _lib.call("ct_iterfdk_err", _tptr(pic), _tptr(out), _np_ptr(beta), len(beta), _np_ptr(U), len(U), _np_ptr(P),
              len(P), _np_ptr(G), len(G), _np_ptr(size), nt, ns, nz, float(D), int(t), _stream())
    return out


def fdkui_filter(R: torch.Tensor, xi, gama, beta, b0: float, fan: float, D: float, ds2d: float, out=None):
    """Curved-detector FDK filter stage on the device: R float64 [beta][xi][gamma]
    -> weighted, filtered rows as float32 (ct_fdkui_filter)."""
    if R.dtype != torch.float64 or not R.is_cuda or not R.is_contiguous():
        raise ValueError("R must be a contiguous float64 CUDA tensor")
    nb, lx, lg = R.shape
    xi, gama, beta = (np.ascontiguousarray(a, np.float64) for a in (xi, gama, beta))
    out = torch.empty(R.shape, dtype=torch.float32, device=R.device) if out is None else out
    _lib.call("ct_fdkui_filter", C.c_void_p(R.data_ptr()), _tptr(out), _np_ptr(xi), _np_ptr(gama), _np_ptr(beta),
              float(b0), float(fan), float(D), float(ds2d), lg, nb, lx, _stream())
    return out


def fdkui_bp(rcov: torch.Tensor, xi, gama, beta, D: float, ds2d: float, size, z_length: int, out=None):
    """Curved-detector FDK backprojection of float32 rcov [beta][xi][gamma] into a
    float64 display [z][s][t] (ct_fdkui_bp)."""
    nb, lx, lg = rcov.shape
    xi, gama, beta = (np.ascontiguousarray(a, np.float64) for a in (xi, gama, beta))
    size = np.ascontiguousarray(size, np.int32)
    if out is None:
        out = torch.empty((int(z_length), int(size[1]), int(size[0])), dtype=torch.float64, device=rcov.device)
    _lib.call("ct_fdkui_bp", _tptr(rcov), C.c_void_p(out.data_ptr()), _np_ptr(xi), _np_ptr(gama), _np_ptr(beta),
              float(D), float(ds2d), lg, nb, lx, _np_ptr(size), int(z_length), _stream())
    return out


def tv_flow(x: torch.Tensor, iters: int, step: float, eps: float = 1e-8, lo: float = 0.0, work=None, scratch=None):
    """Normalised isotropic TV gradient-flow sub-iterations on x ([nz][ny][nx] or [ny][nx]), in place."""
    if x.dim() == 2:
        nz, (ny, nx) = 1, x.shape
    else:
        nz, ny, nx = x.shape
    work = torch.empty_like(x) if work is None else work
    scratch = torch.zeros(2, dtype=torch.float64, device=x.device) if scratch is None else scratch
    _lib.call("ct_tv_flow", _tptr(x), _tptr(work), _tptr(scratch), nx, ny, nz, int(iters), float(step), float(eps),
              float(lo), _stream())
    return x


def tv_flow_asd(x: torch.Tensor, prev: torch.Tensor, work: torch.Tensor, scratch: torch.Tensor, state: torch.Tensor,
                iters: int, eps: float = 1e-8, lo: float = 0.0, alpha_red: float = 0.95, r_max: float = 0.95):
    """The TV phase of one ASD-POCS iteration on the device (ct_tv_flow_asd);
    prev = x before the data step on entry, x after it on return; state =
    float64 [alpha, -, -]."""
    nz, ny, nx = x.shape if x.dim() == 3 else (1, *x.shape)
    _lib.call("ct_tv_flow_asd", _tptr(x), _tptr(prev), _tptr(work), _tptr(scratch), _tptr(state), nx, ny, nz,
              int(iters), float(eps), float(lo), float(alpha_red), float(r_max), _stream())
    return x


def sq_diff_sum(a: torch.Tensor, b: torch.Tensor, out: torch.Tensor | None = None) -> torch.Tensor:
    out = torch.zeros(1, dtype=torch.float64, device=a.device) if out is None else out
    _lib.call("ct_sq_diff_sum", _tptr(a), _tptr(b), int(a.numel()), _tptr(out), _stream())
    return out
