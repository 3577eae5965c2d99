"""Host logic of the splits in model3d_gb300/shard.py, on CPU: the
largest-first partition, the slab ranges, and the merge of z-slab meshes --
checked with slab meshes from the oracle (whose z-range option meshes the
same cube layers), in one process and across two gloo ranks that each mesh
their own slab and gather to rank 0.
"""
import os

import numpy as np
import pytest

from model3d_gb300 import Mesh, canonical, serialize
from model3d_gb300.shard import merge_slabs, partition_jobs, slab_ranges
from model3d_gb300.workloads import csg_tree


def test_partition_is_largest_first_and_complete():
    costs = [5, 1, 9, 3, 3, 7, 2, 8]
    parts = partition_jobs(costs, 3)
    assert sorted(i for p in parts for i in p) == list(range(len(costs)))
    loads = sorted(sum(costs[i] for i in p) for p in parts)
    assert loads == [12, 13, 13]  # 9+3 | 8+3+2 | 7+5+1
    assert partition_jobs(costs, 1) == [list(range(len(costs)))]
    assert partition_jobs([], 4) == [[], [], [], []]
    with pytest.raises(ValueError):
        partition_jobs(costs, 0)


def test_slab_ranges():
    assert slab_ranges(10, 3) == [(0, 3), (3, 6), (6, 10)]
    assert slab_ranges(2, 5) == [(0, 1), (1, 2)]
    assert slab_ranges(7, 1) == [(0, 7)]
    for n in (1, 5, 64, 101):
        for p in (1, 2, 3, 8):
            r = slab_ranges(n, p)
            assert r[0][0] == 0 and r[-1][1] == n
            assert all(a < b for a, b in r) and all(r[i][1] == r[i + 1][0] for i in range(len(r) - 1))


def _indexed(soup):
    """Indexed mesh of a (T, 9) triangle soup (unique vertices by bits)."""
    if len(soup) == 0:
        return Mesh(np.zeros((0, 3)), np.zeros((0, 3), dtype=np.int32))
    pts = np.ascontiguousarray(soup.reshape(-1, 3))
    u, inv = np.unique(pts.view(np.dtype((np.void, 24))).ravel(), return_inverse=True)
    verts = np.frombuffer(u.tobytes(), dtype=np.float64).reshape(-1, 3).copy()
    return Mesh(verts, inv.reshape(-1, 3).astype(np.int32))


def _oracle_slab(oracle, nodes, sets, delta, iters, a, b):
    """The oracle's mesh of cube layers [a, b): corner planes a..b."""
    return _indexed(oracle.mc_search(nodes, sets, delta, iters, z_range=(a, b + 1))["tris"])


@pytest.mark.parametrize("parts", [2, 5])
def test_merge_of_oracle_slabs_is_the_whole_mesh(oracle, parts):
    solid = csg_tree(3, 12, 4)
    nodes, sets = serialize(solid)
    whole = oracle.mc_search(nodes, sets, 0.03, 8)
    zs = oracle.spacer_axis(solid.Min().Z, solid.Max().Z, 0.03)
    ranges = slab_ranges(len(zs) - 1, parts)
    meshes = [_oracle_slab(oracle, nodes, sets, 0.03, 8, a, b) for a, b in ranges]
    merged = merge_slabs(meshes, [zs[b] for _, b in ranges[:-1]])
    assert np.array_equal(canonical(merged.TriangleSoup()), canonical(whole["tris"]))
    assert len(merged.vertices) == whole["n_vertices"]


def test_merge_refuses_slabs_that_disagree(oracle):
    solid = csg_tree(3, 12, 4)
    nodes, sets = serialize(solid)
    zs = oracle.spacer_axis(solid.Min().Z, solid.Max().Z, 0.03)
    ranges = slab_ranges(len(zs) - 1, 2)
    meshes = [_oracle_slab(oracle, nodes, sets, 0.03, 8, a, b) for a, b in ranges]
    (a, b) = ranges[0]
    on_plane = np.nonzero(meshes[0].vertices[:, 2] == zs[b])[0]
    assert len(on_plane)
    meshes[0].vertices[on_plane[0], 0] = np.nextafter(meshes[0].vertices[on_plane[0], 0], 9.0)
    with pytest.raises(RuntimeError):
        merge_slabs(meshes, [zs[b]])


def _rank_main(rank, world, port, q):
    import torch.distributed as dist
    os.environ.update(MASTER_ADDR="127.0.0.1", MASTER_PORT=str(port))
    dist.init_process_group("gloo", rank=rank, world_size=world)
    try:
        from oracle import oracle as O
        from model3d_gb300.shard import gather_to_rank0
        solid = csg_tree(3, 12, 4)
        nodes, sets = serialize(solid)
        zs = O.spacer_axis(solid.Min().Z, solid.Max().Z, 0.03)
        ranges = slab_ranges(len(zs) - 1, world)
        a, b = ranges[rank]
        mine = _oracle_slab(O, nodes, sets, 0.03, 8, a, b)
        got = gather_to_rank0((mine.vertices, mine.triangles), rank, world)
        if rank == 0:
            merged = merge_slabs([Mesh(v, t) for v, t in got], [zs[e] for _, e in ranges[:-1]])
            whole = O.mc_search(nodes, sets, 0.03, 8)
            q.put(bool(np.array_equal(canonical(merged.TriangleSoup()), canonical(whole["tris"]))))
    finally:
        dist.destroy_process_group()


def test_two_gloo_ranks_mesh_their_slabs_and_merge_on_rank0():
    import multiprocessing as mp
    import socket
    ctx = mp.get_context("spawn")
    with socket.socket() as s:
        s.bind(("127.0.0.1", 0))
        port = s.getsockname()[1]
    q = ctx.Queue()
    procs = [ctx.Process(target=_rank_main, args=(r, 2, port, q)) for r in range(2)]
    for p in procs:
        p.start()
    for p in procs:
        p.join(120)
    assert all(p.exitcode == 0 for p in procs)
    assert q.get(timeout=5) is True
