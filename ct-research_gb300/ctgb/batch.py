"""Batched SIRT over many 2D fan slices of uneven size (ct_fan_batch_*).

All slices advance together: one forward-projection launch and one
backprojection launch per iteration cover every slice (fan_batch.cu), and a
whole run of `iters` iterations is captured once into a CUDA graph, so the
reconstruction is a single graph launch.  The block sizes of the two launches
come from `autotune`, which times the candidates on the batch itself and
caches the choice per GPU model and batch signature.

Per slice the update is SIRT.m's (lam 2, x in [0, 1], MATLAB eps, optional
FBPfan start; see ctgb.sirt).
"""
from __future__ import annotations

import ctypes as C
import hashlib
import json
import os
from pathlib import Path

import numpy as np
import torch

from . import _lib
from .geometry import FanGeometry
from .sirt import MATLAB_EPS

_CACHE = Path(__file__).resolve().parent / "_lib" / "autotune.json"
FP_BLOCKS = (64, 128, 256)
BP_BLOCKS = (64, 128, 256, 512)


def _stream():
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


def _p(t):
    return C.c_void_p(t.data_ptr())


class FanBatch:
    """Packed operators over a list of FanGeometry slices."""

    def __init__(self, geoms: list[FanGeometry]):
        self.geoms = list(geoms)
        n = len(self.geoms)
        nt = np.array([g.nt for g in self.geoms], np.int32)
        ns = np.array([g.ns for g in self.geoms], np.int32)
        size = np.array([s for g in self.geoms for s in g.size], np.float64)
        nb = np.array([len(g.beta) for g in self.geoms], np.int32)
        npd = np.array([len(g.P) for g in self.geoms], np.int32)
        D = np.array([g.D for g in self.geoms], np.float64)
        betas = [np.ascontiguousarray(g.beta, np.float64) for g in self.geoms]
        Ps = [np.ascontiguousarray(g.P, np.float64) for g in self.geoms]
        bptr = (C.c_void_p * n)(*[b.ctypes.data for b in betas])
        pptr = (C.c_void_p * n)(*[p.ctypes.data for p in Ps])
        self._keep = (nt, ns, size, nb, npd, D, betas, Ps, bptr, pptr)
        self._h = C.c_void_p()
        _lib.call("ct_fan_batch_create", C.byref(self._h), n, nt.ctypes.data_as(C.c_void_p),
                  ns.ctypes.data_as(C.c_void_p), size.ctypes.data_as(C.c_void_p), C.cast(bptr, C.c_void_p),
                  nb.ctypes.data_as(C.c_void_p), C.cast(pptr, C.c_void_p), npd.ctypes.data_as(C.c_void_p),
                  D.ctypes.data_as(C.c_void_p))
        self.blocks = (128, 128)
        self._layout()

    def _layout(self):
        n = len(self.geoms)
        io = np.zeros(n + 1, np.int64)
        so = np.zeros(n + 1, np.int64)
        _lib.call("ct_fan_batch_layout", self._h, io.ctypes.data_as(C.c_void_p), so.ctypes.data_as(C.c_void_p))
        self.img_off, self.sino_off = io, so

    def close(self):
        if self._h:
            _lib.lib().ct_fan_batch_destroy(self._h)
            self._h = C.c_void_p()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    @property
    def n_img(self):
        return int(self.img_off[-1])

    @property
    def n_sino(self):
        return int(self.sino_off[-1])

    @property
    def n_rays(self):
        return self.n_sino

    def set_filter(self, kind="shepp-logan", window: int = 0, short_scan: bool = False):
        """FBP filter options of every slice (FanPlan.set_filter)."""
        from .device import filter_kind
        _lib.call("ct_fan_batch_set_filter", self._h, filter_kind(kind), int(window), int(bool(short_scan)))
        return self

    def set_blocks(self, fp_block: int, bp_block: int):
        _lib.call("ct_fan_batch_set_blocks", self._h, int(fp_block), int(bp_block))
        self.blocks = (int(fp_block), int(bp_block))
        self._layout()

    # packing helpers ---------------------------------------------------------
    def pack_images(self, imgs, device="cuda"):
        out = torch.empty(self.n_img, dtype=torch.float32, device=device)
        for k, im in enumerate(imgs):
            out[self.img_off[k]:self.img_off[k + 1]] = torch.as_tensor(im, dtype=torch.float32).reshape(-1)
        return out

    def pack_sinos(self, sinos, device="cuda"):
        out = torch.empty(self.n_sino, dtype=torch.float32, device=device)
        for k, s in enumerate(sinos):
            out[self.sino_off[k]:self.sino_off[k + 1]] = torch.as_tensor(s, dtype=torch.float32).reshape(-1)
        return out

    def image(self, packed, k):
        g = self.geoms[k]
        return packed[self.img_off[k]:self.img_off[k + 1]].reshape(g.img_shape)

    def sino(self, packed, k):
        g = self.geoms[k]
        return packed[self.sino_off[k]:self.sino_off[k + 1]].reshape(g.sino_shape)

    # operators -----------------------------------------------------------------
    def fp(self, img, out=None):
        out = torch.empty(self.n_sino, dtype=torch.float32, device=img.device) if out is None else out
        _lib.call("ct_fan_batch_fp", self._h, _p(img), _p(out), _stream())
        return out

    def bp(self, proj, out=None):
        out = torch.empty(self.n_img, dtype=torch.float32, device=proj.device) if out is None else out
        _lib.call("ct_fan_batch_bp", self._h, _p(proj), _p(out), _stream())
        return out

    def fp_residual(self, img, b, rowsum, eps, out, norms):
        _lib.call("ct_fan_batch_fp_residual", self._h, _p(img), _p(b), _p(rowsum) if rowsum is not None else None,
                  float(eps), _p(out), _p(norms), _stream())

    def bp_update(self, proj, colsum, img, lam, eps, lo, hi):
        _lib.call("ct_fan_batch_bp_update", self._h, _p(proj), _p(colsum), float(eps), float(lam), float(lo),
                  float(hi), _p(img), _stream())

    def fbp(self, proj, out=None, filter_mode=1):
        out = torch.empty(self.n_img, dtype=torch.float32, device=proj.device) if out is None else out
        _lib.call("ct_fan_batch_fbp", self._h, _p(proj), _p(out), int(filter_mode), _stream())
        return out

    def grazing_rays(self) -> int:
        """Rays of the last forward projection that took the FP64 re-walk."""
        n = C.c_longlong()
        _lib.call("ct_fan_batch_grazing_rays", self._h, C.byref(n), _stream())
        return int(n.value)

    def signature(self) -> str:
        h = hashlib.sha1()
        for g in self.geoms:
            h.update(np.array([g.nt, g.ns, len(g.beta), len(g.P)], np.int64).tobytes())
        return h.hexdigest()[:16]


class BatchedSirt:
    """SIRT of every slice of a FanBatch; a run is one CUDA-graph launch."""

    def __init__(self, batch: FanBatch, b, lam=2.0, lo=0.0, hi=1.0, eps=MATLAB_EPS):
        self.batch, self.b = batch, b
        self.lam, self.lo, self.hi, self.eps = lam, lo, hi, eps
        dev = b.device
        self.rowsum = batch.fp(torch.ones(batch.n_img, dtype=torch.float32, device=dev))
        self.colsum = batch.bp(torch.ones(batch.n_sino, dtype=torch.float32, device=dev))
        self.e = torch.empty_like(b)

    def _iterate(self, x, norms):
        self.batch.fp_residual(x, self.b, self.rowsum, self.eps, self.e, norms)
        self.batch.bp_update(self.e, self.colsum, x, self.lam, self.eps, self.lo, self.hi)

    def capture(self, x, iters: int):
        """Capture `iters` iterations on packed x into one CUDA graph; returns
        (graph, norms) with norms[i] the per-slice sums of iteration i."""
        nsl = len(self.batch.geoms)
        norms = torch.zeros(iters, nsl, 2, dtype=torch.float64, device=x.device)
        # first call allocates the graze list; keep it out of the capture
        warm = x.clone()
        self._iterate(warm, torch.zeros(nsl, 2, dtype=torch.float64, device=x.device))
        torch.cuda.synchronize()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g):
            for i in range(iters):
                self._iterate(x, norms[i])
        return g, norms

    @staticmethod
    def history(norms):
        n = norms.cpu().numpy()
        return np.sqrt(n[..., 0] / np.maximum(n[..., 1], 1e-300))

    def run(self, x, iters: int, graph: bool = True):
        """Run `iters` iterations in place on packed x.  Returns the residual
        history [iters, slices] (relative residual of the x entering each)."""
        if graph:
            g, norms = self.capture(x, iters)
            self.graph = g
            g.replay()
        else:
            norms = torch.zeros(iters, len(self.batch.geoms), 2, dtype=torch.float64, device=x.device)
            for i in range(iters):
                self._iterate(x, norms[i])
        torch.cuda.synchronize()
        return self.history(norms)


def _load_cache():
    try:
        return json.loads(_CACHE.read_text())
    except Exception:
        return {}


def autotune(batch: FanBatch, b, reps: int = 2, use_cache: bool = True):
    """Pick the (fp_block, bp_block) pair with the fastest SIRT iteration on
    this batch; the choice is cached per GPU model and batch signature."""
    key = f"{torch.cuda.get_device_name()}|{batch.signature()}"
    cache = _load_cache()
    if use_cache and key in cache:
        fb, bb = cache[key]["blocks"]
        batch.set_blocks(fb, bb)
        return cache[key]
    sirt = BatchedSirt(batch, b)
    x = torch.zeros(batch.n_img, dtype=torch.float32, device=b.device)
    norms = torch.zeros(len(batch.geoms), 2, dtype=torch.float64, device=b.device)
    timings = {}
    for fb in FP_BLOCKS:
        for bb in BP_BLOCKS:
            batch.set_blocks(fb, bb)
            sirt._iterate(x, norms)
            ev0, ev1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            ev0.record()
            for _ in range(reps):
                sirt._iterate(x, norms)
            ev1.record()
            torch.cuda.synchronize()
            timings[f"{fb},{bb}"] = ev0.elapsed_time(ev1) / reps
    best = min(timings, key=timings.get)
    fb, bb = (int(v) for v in best.split(","))
    batch.set_blocks(fb, bb)
    entry = {"blocks": [fb, bb], "ms_per_iteration": timings[best], "candidates": timings}
    cache[key] = entry
    try:
        _CACHE.parent.mkdir(parents=True, exist_ok=True)
        tmp = _CACHE.with_suffix(".tmp")
        tmp.write_text(json.dumps(cache, indent=1))
        os.replace(tmp, _CACHE)
    except OSError:
        pass
    return entry
