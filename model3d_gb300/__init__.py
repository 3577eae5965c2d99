"""model3d_gb300 — GB300-native MarchingCubesSearch for model3d solids.

The reference-facing names (Sphere, Cylinder, JoinedSolid, TransformSolid,
MeshToCollider, NewColliderSolid, MarchingCubesSearch, ...) mirror package
model3d of unixpickle/model3d (metaball solids included).  Containment, cube classification, vertex
dedup and the bisection search run in CUDA kernels for sm_103a
(model3d_gb300/csrc); results are bit-identical to the reference algorithm.
"""
from .geometry import Coord3D, Matrix3, NewMatrix3Rotation, X, XYZ, Y, Z
from .solids import (Capsule, CacheSolidBounds, ColliderSolid, Cylinder, ForceSolidBounds,
                     GroupBounders, GroupedTrianglesToCollider, IntersectedSolid, JoinedSolid,
                     JoinedTransform, Matrix3Transform, MeshToCollider, NewColliderSolid,
                     NewRect, NotLowerable, Rect, RotateSolid, Rotation, Scale, ScaleSolid,
                     Solid, Sphere, Subtract, SubtractedSolid, Torus, TransformSolid, Translate,
                     TranslateSolid, VecScale, VecScaleSolid, serialize)
from .metaballs import (CubicMetaballFalloffFunc, ExponentialMetaballFalloffFunc,
                        GaussianMetaballFalloffFunc, InversePowerMetaballFalloffFunc,
                        LinearMetaballFalloffFunc, MetaballSolid, QuadraticMetaballFalloffFunc,
                        QuarticMetaballFalloffFunc, QuinticMetaballFalloffFunc, RotateMetaball,
                        ScaleMetaball, SDFToMetaball, SignedMetaballSolid, TransformMetaball,
                        TranslateMetaball, VecScaleMetaball, WeightedMetaballSolid,
                        WyvillMetaballFalloffFunc)
from .mc import (Context, Contains, DeviceSolid, GroupTriangles, MarchingCubes, MarchingCubesConj,
                 MarchingCubesInterior, MarchingCubesSearch, MarchingCubesSearchBatch,
                 MarchingCubesSearchGroupedSTL, MarchingCubesSearchSTL, MCError,
                 Mesh, autotune, canonical, case_table, check_program, default_context, measure_peaks,
                 spacer_axis)

from .filter import MarchingCubesC2F, MarchingCubesFilter, MarchingCubesSearchFilter, RectCollider

__all__ = [n for n in dir() if not n.startswith("_")]
