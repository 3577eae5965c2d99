"""Seeded synthetic workloads with the shapes of the benchmark configurations.

No public dataset is involved: every input is generated from a splitmix64
stream with a fixed seed, so the oracle and the GPU see identical bytes.

  csg_tree(seed, 48, 16)   JoinedSolid of 48 primitives minus a JoinedSolid of
                           16; kinds uniform over Sphere/Cylinder/Rect/Capsule,
                           centres U[-1,1]^3, radii / half-extents /
                           half-lengths U[0.05,0.3], axes random unit vectors.
  displaced_icosphere(n)   icosahedron with every face split n x n (20 n^2
                           triangles), projected to the unit sphere and
                           displaced radially by r = 1 + 0.15 * (sum of 8
                           sinusoids sin(f_k * (u_k . p) + phi_k)), f_k in
                           1..6, u_k random unit vectors, phi_k U[0, 2 pi);
                           r is kept >= 0.2 (the guard never binds for the
                           seeds used here: r stays within about [0.4, 1.9]).
                           A radial graph with r > 0 cannot self-intersect.
  metaball_blob(seed, n)   MetaballSolid of n balls, 3/4 spheres and 1/4
                           capsules: centres U[-0.7,0.7]^3, radii U[0.05,0.2],
                           capsule half-lengths U[0.05,0.25] along random unit
                           axes; quartic falloff, radiusThreshold 0.1.
"""
from __future__ import annotations

import math
from typing import List, Tuple

import numpy as np

from .geometry import XYZ, Coord3D
from .solids import (Capsule, Cylinder, JoinedSolid, Rect, Sphere, Solid, SubtractedSolid)
from .metaballs import MetaballSolid

_M64 = (1 << 64) - 1


class SplitMix64:
    """splitmix64 (Steele, Lea, Flood 2014): state += 0x9e3779b97f4a7c15, then
    two xor-shift-multiply rounds."""

    def __init__(self, seed: int):
        self.s = seed & _M64

    def next_u64(self) -> int:
        self.s = (self.s + 0x9E3779B97F4A7C15) & _M64
        z = self.s
        z = ((z ^ (z >> 30)) * 0xBF58476D1CE4E5B9) & _M64
        z = ((z ^ (z >> 27)) * 0x94D049BB133111EB) & _M64
        return z ^ (z >> 31)

    def uniform(self, lo: float = 0.0, hi: float = 1.0) -> float:
        return lo + (hi - lo) * ((self.next_u64() >> 11) * (1.0 / (1 << 53)))

    def unit_vector(self) -> Coord3D:
        while True:
            v = [self.uniform(-1, 1) for _ in range(3)]
            n = math.sqrt(sum(x * x for x in v))
            if 1e-3 < n <= 1:
                return XYZ(v[0] / n, v[1] / n, v[2] / n)

    def log_uniform(self, lo: float, hi: float) -> float:
        return math.exp(self.uniform(math.log(lo), math.log(hi)))


def random_primitive(rng: SplitMix64) -> Solid:
    kind = rng.next_u64() % 4
    c = XYZ(rng.uniform(-1, 1), rng.uniform(-1, 1), rng.uniform(-1, 1))
    if kind == 0:
        return Sphere(c, rng.uniform(0.05, 0.3))
    if kind == 1:
        h = XYZ(rng.uniform(0.05, 0.3), rng.uniform(0.05, 0.3), rng.uniform(0.05, 0.3))
        return Rect(c.Sub(h), c.Add(h))
    axis = rng.unit_vector()
    half = rng.uniform(0.05, 0.3)
    r = rng.uniform(0.05, 0.3)
    p1, p2 = c.Add(axis.Scale(half)), c.Sub(axis.Scale(half))
    return Cylinder(p1, p2, r) if kind == 2 else Capsule(p1, p2, r)


def csg_tree(seed: int, n_pos: int = 48, n_neg: int = 16) -> Solid:
    """SubtractedSolid{JoinedSolid(n_pos primitives), JoinedSolid(n_neg)}."""
    rng = SplitMix64(seed)
    pos = [random_primitive(rng) for _ in range(n_pos)]
    if n_neg == 0:
        return JoinedSolid(pos)
    neg = [random_primitive(rng) for _ in range(n_neg)]
    return SubtractedSolid(JoinedSolid(pos), JoinedSolid(neg))


def csg_batch(seed: int, count: int = 512, grid_lo: int = 32, grid_hi: int = 384,
              n_lo: int = 4, n_hi: int = 128) -> List[Tuple[Solid, float]]:
    """(solid, delta) pairs: N log-uniform primitives (3/4 joined, 1/4
    subtracted), delta chosen so the grid's longest side is log-uniform."""
    rng = SplitMix64(seed)
    out = []
    for i in range(count):
        n = int(round(rng.log_uniform(n_lo, n_hi)))
        n_neg = max(0, n // 4)
        solid = csg_tree(rng.next_u64(), n - n_neg, n_neg)
        side = rng.log_uniform(grid_lo, grid_hi)
        mn, mx = solid.Min(), solid.Max()
        ext = max(mx.X - mn.X, mx.Y - mn.Y, mx.Z - mn.Z)
        out.append((solid, ext / (side - 3)))
    return out


def collider_batch(seed: int, count: int = 64, tri_lo: int = 20000, tri_hi: int = 2000000,
                   grid_lo: int = 128, grid_hi: int = 512) -> List[Tuple[np.ndarray, int, int]]:
    """(triangles, seed, grid side) of displaced icospheres: triangle counts
    log-uniform in [tri_lo, tri_hi] (an icosphere has 20 n^2 triangles, so n is
    rounded), each meshed at a grid whose longest side is log-uniform in
    [grid_lo, grid_hi] corners; delta = extent / (side - 3)."""
    rng = SplitMix64(seed)
    out = []
    for i in range(count):
        t = rng.log_uniform(tri_lo, tri_hi)
        n = max(1, int(round(math.sqrt(t / 20))))
        mesh_seed = int(rng.next_u64() % (1 << 31))
        side = int(round(rng.log_uniform(grid_lo, grid_hi)))
        out.append((displaced_icosphere(n, mesh_seed), mesh_seed, side))
    return out


def metaball_blob(seed: int, n: int = 64, falloff=None, radius_threshold: float = 0.1) -> Solid:
    """MetaballSolid(falloff, radius_threshold, n balls) (falloff None: quartic)."""
    rng = SplitMix64(seed)
    balls = []
    for _ in range(n):
        c = XYZ(rng.uniform(-0.7, 0.7), rng.uniform(-0.7, 0.7), rng.uniform(-0.7, 0.7))
        r = rng.uniform(0.05, 0.2)
        if rng.next_u64() % 4 == 0:
            axis = rng.unit_vector()
            half = rng.uniform(0.05, 0.25)
            balls.append(Capsule(c.Add(axis.Scale(half)), c.Sub(axis.Scale(half)), r))
        else:
            balls.append(Sphere(c, r))
    return MetaballSolid(falloff, radius_threshold, *balls)


def icosphere_triangles(n: int) -> np.ndarray:
    """(20 n^2, 9) triangles of an icosahedron with faces split n x n, on the
    unit sphere, counter-clockwise seen from outside."""
    t = (1 + math.sqrt(5)) / 2
    V = np.array([[-1, t, 0], [1, t, 0], [-1, -t, 0], [1, -t, 0], [0, -1, t], [0, 1, t],
                  [0, -1, -t], [0, 1, -t], [t, 0, -1], [t, 0, 1], [-t, 0, -1], [-t, 0, 1]], float)
    F = [(0, 11, 5), (0, 5, 1), (0, 1, 7), (0, 7, 10), (0, 10, 11), (1, 5, 9), (5, 11, 4),
         (11, 10, 2), (10, 7, 6), (7, 1, 8), (3, 9, 4), (3, 4, 2), (3, 2, 6), (3, 6, 8),
         (3, 8, 9), (4, 9, 5), (2, 4, 11), (6, 2, 10), (8, 6, 7), (9, 8, 1)]
    tris = []
    ii, jj = np.meshgrid(np.arange(n), np.arange(n), indexing="ij")
    mask_up = (ii + jj) < n
    mask_dn = (ii + jj) < n - 1
    for a, b, c in F:
        A, B, C = V[a], V[b], V[c]

        def P(i, j):
            return A[None, None] + (B - A)[None, None] * (i[..., None] / n) + \
                (C - A)[None, None] * (j[..., None] / n)

        p0, p1, p2 = P(ii, jj), P(ii + 1, jj), P(ii, jj + 1)
        up = np.concatenate([p0, p1, p2], axis=-1)[mask_up]
        q0, q1, q2 = P(ii + 1, jj), P(ii + 1, jj + 1), P(ii, jj + 1)
        dn = np.concatenate([q0, q1, q2], axis=-1)[mask_dn]
        tris.append(up)
        tris.append(dn)
    T = np.concatenate(tris).reshape(-1, 3, 3)
    T /= np.linalg.norm(T, axis=-1, keepdims=True)
    return T.reshape(-1, 9)


def displaced_icosphere(n: int, seed: int = 7) -> np.ndarray:
    """Icosphere of 20 n^2 triangles with the seeded radial displacement."""
    rng = SplitMix64(seed)
    dirs = np.array([rng.unit_vector().Array() for _ in range(8)])
    freqs = np.array([1 + rng.next_u64() % 6 for _ in range(8)], float)
    phases = np.array([rng.uniform(0, 2 * math.pi) for _ in range(8)])
    T = icosphere_triangles(n).reshape(-1, 3)
    r = 1 + 0.15 * np.sum(np.sin(freqs[None] * (T @ dirs.T) + phases[None]), axis=1)
    r = np.maximum(r, 0.2)
    return (T * r[:, None]).reshape(-1, 9)


def box_triangles(mn, mx) -> np.ndarray:
    """12 triangles of an axis-aligned box (two per face, outward winding)."""
    x0, y0, z0 = mn
    x1, y1, z1 = mx
    P = lambda x, y, z: [x1 if x else x0, y1 if y else y0, z1 if z else z0]
    quads = [
        (P(0, 0, 0), P(1, 0, 0), P(1, 0, 1), P(0, 0, 1)),
        (P(1, 1, 1), P(1, 1, 0), P(0, 1, 0), P(0, 1, 1)),
        (P(0, 0, 0), P(0, 0, 1), P(0, 1, 1), P(0, 1, 0)),
        (P(1, 1, 1), P(1, 0, 1), P(1, 0, 0), P(1, 1, 0)),
        (P(0, 0, 0), P(0, 1, 0), P(1, 1, 0), P(1, 0, 0)),
        (P(1, 1, 1), P(0, 1, 1), P(0, 0, 1), P(1, 0, 1)),
    ]
    out = []
    for p1, p2, p3, p4 in quads:  # AddQuad: (p1,p2,p4), (p2,p3,p4)
        out.append(p1 + p2 + p4)
        out.append(p2 + p3 + p4)
    return np.array(out, float)
