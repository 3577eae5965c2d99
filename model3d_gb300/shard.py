"""Splitting MarchingCubesSearch work into independent parts, for several
GPUs (one process per GPU, e.g. under torchrun) or for several calls on one.

The path has no exchange step, so neither split needs a collective on the
device; the parts' meshes are concatenated on the host.

* A batch of solids splits by solid: `partition_jobs` assigns jobs to parts
  largest-first (each to the part with the least work so far), with a job's
  work estimated by its corner count.
* One solid splits into z-slabs: `slab_ranges` cuts the grid's cube layers
  into contiguous ranges and `MarchingCubesSearchSlab` meshes one range
  (mc_opts.z_begin / z_end).  Neighbouring slabs both compute the corner
  plane between them, so both hold the vertices of the x and y edges on that
  plane -- bit-identical, since the spacer, LookupEdgePoint and the solid are
  the whole grid's.  `merge_slabs` keeps one copy (the upper slab's: an edge
  is owned by the slab that holds its lower corner as a first-plane corner)
  and re-indexes the lower slab's triangles.  The merged mesh equals the
  single call's up to the order of vertices and triangles.

The reference meshes one solid in one process: its z-slab ring of goroutines
(model3d/mc.go:614-645) and its concurrent vertex map (mc.go:193-202) are the
within-call analogue of these splits.
"""
from __future__ import annotations

import heapq
from typing import List, Sequence, Tuple

import numpy as np

from .mc import DeviceSolid, Mesh, MarchingCubesSearch, spacer_axis


def _bounds(solid):
    """Root Min()/Max() as two 3-arrays, of a Solid or a DeviceSolid."""
    if isinstance(solid, DeviceSolid):
        return solid.bounds()
    return np.array(solid.Min().Array()), np.array(solid.Max().Array())


def grid_shape(solid, delta: float) -> Tuple[int, int, int]:
    """(nx, ny, nz) of newSquareSpacer(solid, delta) (model3d/mc.go:594-608)."""
    mn, mx = _bounds(solid)
    return tuple(len(spacer_axis(mn[a], mx[a], delta)) for a in range(3))


def partition_jobs(costs: Sequence[float], parts: int) -> List[List[int]]:
    """Job indices per part, largest job first onto the least-loaded part
    (ties: lower job index first, lower part index first).  Each part's list
    is in ascending job order."""
    if parts < 1:
        raise ValueError("parts must be >= 1")
    order = sorted(range(len(costs)), key=lambda i: (-float(costs[i]), i))
    heap = [(0.0, p) for p in range(parts)]
    out: List[List[int]] = [[] for _ in range(parts)]
    for i in order:
        load, p = heapq.heappop(heap)
        out[p].append(i)
        heapq.heappush(heap, (load + float(costs[i]), p))
    return [sorted(o) for o in out]


def job_costs(jobs) -> List[int]:
    """Corner counts of (solid, delta, iters) jobs (solid or DeviceSolid)."""
    out = []
    for s, d, _ in jobs:
        nx, ny, nz = grid_shape(s, d)
        out.append(nx * ny * nz)
    return out


def slab_ranges(n_layers: int, parts: int) -> List[Tuple[int, int]]:
    """Contiguous cube-layer ranges [z_begin, z_end) covering [0, n_layers),
    sizes differing by at most one; empty parts are dropped."""
    parts = max(1, min(parts, n_layers))
    cuts = [n_layers * p // parts for p in range(parts + 1)]
    return [(a, b) for a, b in zip(cuts, cuts[1:]) if b > a]


def MarchingCubesSearchSlab(solid, delta: float, iters: int, z_begin: int, z_end: int, **kw) -> Mesh:
    """The part of MarchingCubesSearch(solid, delta, iters) in cube layers
    [z_begin, z_end) of the solid's grid."""
    return MarchingCubesSearch(solid, delta, iters, z_range=(z_begin, z_end), **kw)


def _plane_rows(v: np.ndarray, z: float) -> np.ndarray:
    """Indices of the vertices on the corner plane z, sorted by their (x, y)
    bit patterns."""
    idx = np.nonzero(v[:, 2] == z)[0]
    bits = np.ascontiguousarray(v[idx, :2]).view(np.uint64)
    return idx[np.lexsort((bits[:, 1], bits[:, 0]))]


def merge_slabs(meshes: Sequence[Mesh], planes: Sequence[float]) -> Mesh:
    """One mesh from the meshes of consecutive z-slabs; planes[i] is the z
    value of the corner plane shared by slabs i and i + 1."""
    if len(planes) != max(0, len(meshes) - 1):
        raise ValueError("need one shared plane between consecutive slabs")
    n = len(meshes)
    drop = [np.zeros(len(m.vertices), dtype=bool) for m in meshes]
    link = [None] * n  # (lower-slab rows, upper-slab rows) of the shared plane above slab i
    for i, z in enumerate(planes):
        lo, hi = _plane_rows(meshes[i].vertices, z), _plane_rows(meshes[i + 1].vertices, z)
        a, b = meshes[i].vertices[lo], meshes[i + 1].vertices[hi]
        if a.shape != b.shape or not np.array_equal(a.view(np.uint64), b.view(np.uint64)):
            raise RuntimeError(f"slabs {i} and {i + 1} disagree on their shared plane")
        drop[i][lo] = True
        link[i] = (lo, hi)
    # New index of every kept vertex, slab by slab.
    new_index, base = [], 0
    for i, m in enumerate(meshes):
        keep = ~drop[i]
        ni = np.full(len(m.vertices), -1, dtype=np.int64)
        ni[keep] = base + np.arange(int(keep.sum()))
        base += int(keep.sum())
        new_index.append(ni)
    for i in range(n - 2, -1, -1):  # dropped rows point at the upper slab's copy
        lo, hi = link[i]
        new_index[i][lo] = new_index[i + 1][hi]
    verts = np.concatenate([m.vertices[~drop[i]] for i, m in enumerate(meshes)]) if n else np.zeros((0, 3))
    tris = np.concatenate([new_index[i][m.triangles] for i, m in enumerate(meshes)]) if n else np.zeros((0, 3))
    stats = {"slabs": n, "vertices": len(verts), "triangles": len(tris)}
    return Mesh(np.ascontiguousarray(verts), np.ascontiguousarray(tris, dtype=np.int32), stats)


def MarchingCubesSearchSlabs(solid, delta: float, iters: int, parts: int, **kw) -> Mesh:
    """MarchingCubesSearch as `parts` z-slab calls, one after another, merged."""
    nx, ny, nz = grid_shape(solid, delta)
    ranges = slab_ranges(max(nz - 1, 0), parts)
    if len(ranges) <= 1:
        return MarchingCubesSearch(solid, delta, iters, **kw)
    mn, mx = _bounds(solid)
    zs = spacer_axis(mn[2], mx[2], delta)
    meshes = [MarchingCubesSearchSlab(solid, delta, iters, a, b, **kw) for a, b in ranges]
    return merge_slabs(meshes, [zs[b] for _, b in ranges[:-1]])


def gather_to_rank0(obj, rank: int, world: int):
    """torch.distributed.gather_object of obj to rank 0 (any backend); the
    list of all ranks' objects on rank 0, None elsewhere."""
    if world == 1:
        return [obj]
    import torch.distributed as dist
    out = [None] * world if rank == 0 else None
    dist.gather_object(obj, out, dst=0)
    return out
