"""Sharding of the product over ranks, on CPU (gloo, world size 2).

The reference spreads lattice blocks over a 2-D MPI process grid and sums
the ranks' partial row sums by a row reduce and a column broadcast
(m_HACApK_solve.f90:278-314).  Here the leaves are dealt to the ranks by
hbi_partition_leaves (host only, in libhbigpu); each rank multiplies its own
leaves (on a GPU: hbi_construct_lh_part; in this CPU test: the oracle's
product of the same leaves, standing in for the device) and one all-reduce
of the N-vector sums the partials.  Checked: the partition covers every leaf
once with balanced factor bytes, and the all-reduced product equals the
one-rank product.
"""
import os
import socket

import numpy as np
import pytest

import hbi_gb300 as H


def _port():
    s = socket.socket()
    s.bind(("127.0.0.1", 0))
    p = s.getsockname()[1]
    s.close()
    return p


def _system(oracle):
    from hbi_gb300 import mesh
    n = 600
    xel, xer, xcol, _ = mesh.mesh_2dp(n, 40.0 / n)
    g = oracle.Geometry(oracle.ORC_2DVS, n, "s", xcol=xcol, xel=xel, xer=xer)
    coord = np.stack([xcol, np.zeros(n), np.zeros(n)], 1)
    lod, lv, _ = oracle.build_structure(coord)
    p = oracle.default_params()
    p[70] = 1e-6
    return n, oracle.HMatrix(g, lod, lv, p)


def _sub(oracle, Ho, keep):
    """The oracle H-matrix of the leaves in `keep` (same packing)."""
    leaves = Ho.leaves[keep]
    parts, off = [], [0]
    for ip in np.nonzero(keep)[0]:
        seg = Ho.body[Ho.off[ip]:Ho.off[ip + 1]]
        parts.append(seg)
        off.append(off[-1] + seg.size)
    body = np.concatenate(parts) if parts else np.zeros(0)
    return oracle.HMatrix.from_body(Ho.n, leaves, np.array(off, dtype=np.int64), body)


def test_partition_covers_every_leaf_once_and_balances(oracle):
    n, Ho = _system(oracle)
    elems = np.where(Ho.leaves[:, 0] == 1, Ho.leaves[:, 1] * (Ho.leaves[:, 3] + Ho.leaves[:, 5]),
                     Ho.leaves[:, 3] * Ho.leaves[:, 5])
    for nr in (1, 2, 3, 8):
        owner, load = H.partition_leaves(Ho.leaves, nr)
        assert owner.min() >= 0 and owner.max() < nr
        assert load.sum() == elems.sum()
        for r in range(nr):
            assert load[r] == elems[owner == r].sum()
        # greedy longest-first: no rank exceeds the mean by more than the largest leaf
        assert load.max() - load.mean() <= elems.max()


def _rank(rank, world, port, q):
    import torch
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    from oracle import oracle
    n, Ho = _system(oracle)
    owner, _ = H.partition_leaves(Ho.leaves, world)
    mine = _sub(oracle, Ho, owner == rank)
    u = np.random.default_rng(3).standard_normal(n)
    y = torch.from_numpy(mine.matvec(u))
    dist.all_reduce(y, op=dist.ReduceOp.SUM)
    q.put((rank, y.numpy()))
    dist.destroy_process_group()


def test_sharded_product_equals_one_rank_product(oracle):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    port = _port()
    ps = [ctx.Process(target=_rank, args=(r, 2, port, q)) for r in range(2)]
    for p in ps:
        p.start()
    res = dict(q.get(timeout=120) for _ in ps)
    for p in ps:
        p.join(timeout=60)
        assert p.exitcode == 0
    n, Ho = _system(oracle)
    u = np.random.default_rng(3).standard_normal(n)
    ref = Ho.matvec(u)
    for r in range(2):
        assert np.linalg.norm(res[r] - ref) <= 1e-13 * np.linalg.norm(ref)
    assert np.array_equal(res[0], res[1])
