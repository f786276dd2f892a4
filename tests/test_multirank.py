"""World-size-2 view sharding on CPU ranks (gloo): the sharded projector pair
and SIRT step equal the single-process result.  The operators are the FP64
oracle, so this exercises the sharding and collective logic only."""
import os
import socket

import numpy as np
import pytest
import torch


def _free_port():
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        return s.getsockname()[1]


def test_view_range_partitions_exactly():
    from ctgb.shard import view_range
    for n in (1, 7, 360):
        for w in (1, 2, 3, 8):
            if w > n:
                continue
            ranges = [view_range(n, r, w) for r in range(w)]
            assert ranges[0][0] == 0 and ranges[-1][1] == n
            assert all(ranges[i][1] == ranges[i + 1][0] for i in range(w - 1))
            sizes = [hi - lo for lo, hi in ranges]
            assert max(sizes) - min(sizes) <= 1
    with pytest.raises(ValueError):
        view_range(10, 2, 2)


class _OraclePlan:
    """Cone operators of the oracle behind the plan interface (CPU tensors)."""

    def __init__(self, geom):
        from oracle.oracle import Oracle
        self.o, self.geom = Oracle(nthreads=2), geom

    def fp(self, x, out=None):
        g = self.geom
        return torch.from_numpy(self.o.cone_fp(x.numpy(), g.beta, g.P, g.xi, g.size, g.D))

    def bp(self, y, out=None):
        g = self.geom
        return torch.from_numpy(self.o.cone_bp(y.numpy(), g.beta, g.P, g.xi, g.size, g.D, g.vol_shape))

    def fp_residual(self, x, b, rowsum=None, eps=0.0, out=None, norms=None):
        r = b.double() - self.fp(x).double()
        out.copy_((r / (rowsum.double() + eps)).float())
        norms[0] += float((r * r).sum())
        norms[1] += float((b.double() ** 2).sum())
        return out, norms


def _geom():
    from ctgb.geometry import ConeGeometry, view_angles, centred_domain
    return ConeGeometry(12, 12, 10, (12.0, 12.0, 10.0), view_angles(9), centred_domain(24, 0.8),
                        centred_domain(20, 0.7), 40.0)


def _worker(rank, world, port, result_path):
    import torch.distributed as dist
    os.environ["MASTER_ADDR"] = "127.0.0.1"
    os.environ["MASTER_PORT"] = str(port)
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from ctgb import phantom
    from ctgb.shard import ShardedSirt, local_geometry, view_range, allreduce_sum
    g = _geom()
    vol = phantom.ellipsoids_3d(g.nt, g.ns, g.nz, phantom.ellipsoid_params(6, seed=9))
    full = _OraclePlan(g)
    b = full.fp(vol)
    lo, hi = view_range(len(g.beta), rank, world)
    plan = _OraclePlan(local_geometry(g, rank, world))
    # sharded forward projection: this rank's block of views, no exchange
    fp_local = plan.fp(vol)
    # sharded backprojection: partial volumes summed over ranks
    bp = allreduce_sum(plan.bp(b[lo:hi].contiguous()))
    # the bench's sharded pair: block of the sinogram and the all-reduced A^T A x
    from ctgb.shard import ShardedPair
    pair_proj, pair_back = torch.zeros(hi - lo, *g.sino_shape[1:]), torch.zeros(g.vol_shape)

    class _OutPlan:                    # the oracle plan writing into given outputs, as ConePlan does
        geom = plan.geom

        def fp(self, v, out):
            out.copy_(plan.fp(v))
            return out

        def bp(self, y, out):
            out.copy_(plan.bp(y))
            return out

    ShardedPair(_OutPlan()).step(vol, pair_proj, pair_back)
    x = torch.zeros(g.vol_shape)
    sirt = ShardedSirt(plan, b[lo:hi].contiguous(), lam=1.0)
    r = [sirt.step(x) for _ in range(3)]
    np.savez(f"{result_path}_{rank}.npz", fp=fp_local.numpy(), bp=bp.numpy(), x=x.numpy(), r=np.array(r),
             lo=lo, hi=hi, pair_proj=pair_proj.numpy(), pair_back=pair_back.numpy())
    dist.destroy_process_group()


def test_two_rank_view_sharding_equals_single_process(tmp_path):
    import torch.multiprocessing as mp
    from oracle.oracle import sirt_loop
    port = _free_port()
    mp.spawn(_worker, args=(2, port, str(tmp_path / "r")), nprocs=2, join=True)
    g = _geom()
    from ctgb import phantom
    vol = phantom.ellipsoids_3d(g.nt, g.ns, g.nz, phantom.ellipsoid_params(6, seed=9))
    full = _OraclePlan(g)
    b = full.fp(vol)
    bp_full = full.bp(b).numpy()
    ref_x = sirt_loop(lambda v: full.fp(torch.from_numpy(v.astype(np.float32))).numpy(),
                      lambda y: full.bp(torch.from_numpy(y.astype(np.float32))).numpy(),
                      b.numpy(), np.zeros(g.vol_shape), 3, 1.0, 0.0, np.inf, 1e-9)
    res = [np.load(tmp_path / f"r_{k}.npz") for k in range(2)]
    # the two forward-projection blocks tile the full sinogram
    fp = np.concatenate([res[0]["fp"], res[1]["fp"]])
    assert np.array_equal(fp, b.numpy())
    full_back = full.bp(full.fp(vol)).numpy()
    assert np.array_equal(np.concatenate([res[0]["pair_proj"], res[1]["pair_proj"]]), b.numpy())
    for d in res:
        assert np.linalg.norm(d["pair_back"] - full_back) <= 1e-6 * np.linalg.norm(full_back)
        assert np.linalg.norm(d["bp"] - bp_full) <= 1e-6 * np.linalg.norm(bp_full)
        assert np.linalg.norm(d["x"] - ref_x) <= 1e-5 * np.linalg.norm(ref_x)
    assert np.array_equal(res[0]["x"], res[1]["x"])
    assert np.allclose(res[0]["r"], res[1]["r"])
