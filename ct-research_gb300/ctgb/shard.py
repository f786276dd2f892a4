"""View sharding of the projector pair across ranks (one process per GPU).

The rays of different views are independent, so the forward projection of a
scan splits by views with no exchange; the voxel-driven backprojection sums
over views, so each rank backprojects its views into a partial volume and one
all-reduce (sum) combines them.  A SIRT iteration is then: view-sharded
forward projection and residual, view-sharded backprojection, one all-reduce
of the partial volume (and of the two residual norms), and the same update on
every rank.

With one GPU per process this is data parallelism over views; a run that has
only one GPU uses the plain plans (world size 1 reduces to them).
"""
from __future__ import annotations

import numpy as np


def view_range(n_views: int, rank: int, world: int) -> tuple[int, int]:
    """Contiguous block of views [lo, hi) of `rank`; blocks differ by at most one view."""
    if world < 1 or not (0 <= rank < world):
        raise ValueError("bad rank / world size")
    base, extra = divmod(n_views, world)
    lo = rank * base + min(rank, extra)
    return lo, lo + base + (1 if rank < extra else 0)


def local_geometry(geom, rank: int, world: int):
    """The ConeGeometry / FanGeometry of this rank's views."""
    lo, hi = view_range(len(geom.beta), rank, world)
    g = geom.subset_views(np.arange(lo, hi)) if hasattr(geom, "subset_views") else None
    if g is None:
        from .geometry import FanGeometry
        g = FanGeometry(geom.nt, geom.ns, geom.size, geom.beta[lo:hi], geom.P, geom.D, geom.name)
    return g


def allreduce_sum(t, group=None):
    """In-place sum over ranks (torch.distributed); no-op for a single process."""
    import torch.distributed as dist
    if dist.is_available() and dist.is_initialized() and dist.get_world_size(group) > 1:
        dist.all_reduce(t, op=dist.ReduceOp.SUM, group=group)
    return t


class ShardedPair:
    """One forward + back projection of a scan split by views over the ranks:
    `plan` holds this rank's views (local_geometry).  fp writes this rank's
    block of the sinogram (no exchange); bp backprojects that block into a
    partial volume and one all-reduce (sum) makes every rank hold A^T y of the
    whole scan.  With one rank it is the plain pair."""

    def __init__(self, plan, group=None):
        self.plan, self.group = plan, group

    def step(self, vol, proj, back):
        self.plan.fp(vol, proj)
        self.plan.bp(proj, back)
        allreduce_sum(back, self.group)
        return proj, back


class ShardedSirt:
    """SIRT over view shards: `plan` is this rank's plan over its views (anything
    with fp_residual / bp / fp / geom), `b` its block of the sinogram."""

    def __init__(self, plan, b, lam=1.0, lo=0.0, hi=float("inf"), eps=1e-9, group=None):
        import torch
        self.plan, self.b, self.group = plan, b, group
        self.lam, self.lo, self.hi, self.eps = lam, lo, hi, eps
        shape = plan.geom.vol_shape if hasattr(plan.geom, "vol_shape") else plan.geom.img_shape
        ones = torch.ones(shape, dtype=torch.float32, device=b.device)
        self.rowsum = plan.fp(ones)
        self.colsum = allreduce_sum(plan.bp(torch.ones_like(b)), group)
        self.e = torch.empty_like(b)

    def step(self, x):
        import torch
        norms = torch.zeros(2, dtype=torch.float64, device=x.device)
        self.plan.fp_residual(x, self.b, self.rowsum, self.eps, out=self.e, norms=norms)
        part = self.plan.bp(self.e)
        allreduce_sum(part, self.group)
        allreduce_sum(norms, self.group)
        x.copy_(torch.clamp(x + self.lam * part / (self.colsum + self.eps), self.lo, self.hi))
        return float((norms[0] / norms[1]).sqrt()) if float(norms[1]) > 0 else float("nan")
