"""Metaball solids (model3d/metaball.go, model3d/transform.go:319-414).

WeightedMetaballSolid(f, radiusThreshold, balls, weights) contains c when
sum_i weights[i] * f(balls[i].MetaballField(c)) > f(radiusThreshold), inside a
box that the constructor finds by an outset search; every float64 step of
that search is done here in the reference's order, so the bounds (and the
spacer built from them) are the reference's.

A metaball is one of the primitives (Sphere, Rect, Capsule, Cylinder, Torus,
whose MetaballField is -SDF), SDFToMetaball of one of them, or a
TransformMetaball / VecScaleMetaball of a metaball.

Falloffs: the inverse powers 1/r^k for integer k (math.Pow restated below)
and Wyvill's compact falloff lower to the device.  Exponential and Gaussian
falloffs call Go's math.Exp, which amd64 and arm64 implement in assembly, so
they have no single float64 result to reproduce: they raise NotLowerable.
"""
from __future__ import annotations

import math
import struct
from typing import Optional, Sequence

from .geometry import Coord3D, XYZ
from .solids import (Capsule, Cylinder, JoinedTransform, Matrix3Transform, NotLowerable, Rect,
                     Scale, Solid, Sphere, Torus, Transform, Translate, VecScale, NewRect,
                     OrthoMatrix3Transform)

# MC_FALLOFF_* (include/mcgpu.h).
FALLOFF_POWER, FALLOFF_WYVILL = 1, 2
MAX_POWER = 1 << 20


# ----------------------------------------------------- Go math restated

def _bits(x: float) -> int:
    return struct.unpack("<Q", struct.pack("<d", x))[0]


def _from_bits(b: int) -> float:
    return struct.unpack("<d", struct.pack("<Q", b & 0xFFFFFFFFFFFFFFFF))[0]


_SMALLEST_NORMAL = 2.2250738585072014e-308


def go_ldexp(frac: float, exp: int) -> float:
    """math.Ldexp (Go math/ldexp.go): frac * 2^exp, one rounding for
    subnormal results (scale into range, then multiply by 2^-53)."""
    if frac == 0 or math.isinf(frac) or math.isnan(frac):
        return frac
    if abs(frac) < _SMALLEST_NORMAL:  # normalize
        frac *= float(1 << 52)
        exp -= 52
    x = _bits(frac)
    exp += ((x >> 52) & 0x7FF) - 1023
    if exp < -1075:
        return math.copysign(0.0, frac)
    if exp > 1023:
        return -math.inf if frac < 0 else math.inf
    m = 1.0
    if exp < -1022:
        exp += 53
        m = 1.0 / float(1 << 53)
    x &= ~(0x7FF << 52)
    x |= (exp + 1023) << 52
    return m * _from_bits(x)


def go_pow_int(x: float, y: int) -> float:
    """math.Pow(x, y) for an integer y with 0 < |y| < 2^20 and x > 0 finite
    (Go math/pow.go): x = x1 * 2^xe by Frexp, the product of the x1 powers
    over the bits of |y| by repeated squaring (renormalised to [0.5, 1)),
    one reciprocal for y < 0, then Ldexp."""
    if y == 0 or x == 1:
        return 1.0
    if y == 1:
        return x
    if not (x > 0) or math.isinf(x) or not (0 < abs(y) < MAX_POWER):
        raise ValueError("go_pow_int: x must be positive and finite, 0 < |y| < 2^20")
    a1, ae = 1.0, 0
    x1, xe = math.frexp(x)
    i = abs(y)
    while i != 0:
        if xe < -(1 << 12) or (1 << 12) < xe:
            ae += xe
            break
        if i & 1 == 1:
            a1 *= x1
            ae += xe
        x1 *= x1
        xe <<= 1
        if x1 < 0.5:
            x1 += x1
            xe -= 1
        i >>= 1
    if y < 0:
        a1 = 1 / a1
        ae = -ae
    return go_ldexp(a1, ae)


# ------------------------------------------------------------- falloffs

class MetaballFalloff:
    """A MetaballFalloffFunc (model3d/metaball.go:10-13)."""

    kind = 0
    param = 0.0

    def __call__(self, r: float) -> float:
        raise NotImplementedError


class _InversePower(MetaballFalloff):
    """InversePowerMetaballFalloffFunc (model3d/metaball.go:17-28)."""

    kind = FALLOFF_POWER

    def __init__(self, power: float):
        if not (power > 0):
            raise ValueError("power must be positive")
        self.param = float(power)

    def __call__(self, r: float) -> float:
        if r <= 0:
            return math.inf
        if self.param != int(self.param) or self.param >= MAX_POWER:
            raise NotLowerable("non-integer falloff powers call math.Exp/Log: no device lowering")
        return go_pow_int(r, -int(self.param))


class _Wyvill(MetaballFalloff):
    """WyvillMetaballFalloffFunc (model3d/metaball.go:86-103)."""

    kind = FALLOFF_WYVILL

    def __init__(self, d: float):
        if not (d > 0):
            raise ValueError("d must be positive")
        self.param = float(d)
        self.d2 = self.param * self.param

    def __call__(self, r: float) -> float:
        if r < 0:
            return math.inf
        if r >= self.param:
            return 0.0
        ratio2 = (r * r) / self.d2
        value = 1 - ratio2
        return value * value


class _ExpFalloff(MetaballFalloff):
    def __init__(self, name: str):
        self.name = name

    def __call__(self, r: float) -> float:
        raise NotLowerable(f"{self.name} calls Go's math.Exp (per-architecture assembly): no device lowering")


def InversePowerMetaballFalloffFunc(power: float) -> MetaballFalloff:
    return _InversePower(power)


def WyvillMetaballFalloffFunc(d: float) -> MetaballFalloff:
    return _Wyvill(d)


LinearMetaballFalloffFunc = _InversePower(1)
QuadraticMetaballFalloffFunc = _InversePower(2)
CubicMetaballFalloffFunc = _InversePower(3)
QuarticMetaballFalloffFunc = _InversePower(4)
QuinticMetaballFalloffFunc = _InversePower(5)
ExponentialMetaballFalloffFunc = _ExpFalloff("ExponentialMetaballFalloffFunc")
GaussianMetaballFalloffFunc = _ExpFalloff("GaussianMetaballFalloffFunc")


# ------------------------------------------------------------- metaballs

_PRIMITIVES = (Sphere, Rect, Capsule, Cylinder, Torus)


class _SDFMetaball:
    """SDFToMetaball(s) (model3d/metaball.go:257-272): field -s.SDF(c)."""

    def __init__(self, sdf):
        if not isinstance(sdf, _PRIMITIVES):
            raise NotLowerable(f"SDFToMetaball({type(sdf).__name__}) has no device lowering")
        self.sdf = sdf

    def Min(self):
        return self.sdf.Min()

    def Max(self):
        return self.sdf.Max()


class _TransformedMetaball:
    """TransformMetaball's result (model3d/transform.go:319-358)."""

    def __init__(self, t: Transform, m):
        self.transform, self.wrapped = t, m
        _inverse_distance(t, 1.0)  # t.Inverse() must be a DistTransform
        self.min, self.max = t.ApplyBounds(_ball_min(m), _ball_max(m))

    def Min(self):
        return self.min

    def Max(self):
        return self.max


class _VecScaleMetaball:
    """VecScaleMetaball's result (model3d/transform.go:379-414)."""

    def __init__(self, m, scale: Coord3D):
        mn, mx = _ball_min(m).Mul(scale), _ball_max(m).Mul(scale)
        self.min, self.max = mn.Min(mx), mx.Max(mn)
        self.scale = scale
        self.invMaxScale = 1 / scale.Abs().MaxCoord()
        self.wrapped = m

    def Min(self):
        return self.min

    def Max(self):
        return self.max


def SDFToMetaball(s) -> _SDFMetaball:
    return _SDFMetaball(s)


def TransformMetaball(t: Transform, m):
    return _TransformedMetaball(t, m)


def ScaleMetaball(m, s: float):
    return TransformMetaball(Scale(s), m)


def TranslateMetaball(m, offset: Coord3D):
    return TransformMetaball(Translate(offset), m)


def RotateMetaball(m, axis: Coord3D, angle: float):
    from .solids import Rotation
    return TransformMetaball(Rotation(axis, angle), m)


def VecScaleMetaball(m, scale: Coord3D):
    return _VecScaleMetaball(m, scale)


def _check_ball(m):
    if not isinstance(m, _PRIMITIVES + (_SDFMetaball, _TransformedMetaball, _VecScaleMetaball)):
        raise NotLowerable(f"{type(m).__name__} is not a lowerable Metaball")


def _ball_min(m) -> Coord3D:
    _check_ball(m)
    return m.Min()


def _ball_max(m) -> Coord3D:
    _check_ball(m)
    return m.Max()


def _inverse_distance(t: Transform, d: float) -> float:
    """t.Inverse().(DistTransform).ApplyDistance(d) (transform.go:56, :87,
    :186, :220-229); the reference panics when t's inverse is not a
    DistTransform."""
    if isinstance(t, Translate) or isinstance(t, OrthoMatrix3Transform):
        return d
    if isinstance(t, Scale):
        return d * (1 / t.Scale)
    if isinstance(t, JoinedTransform):
        for sub in reversed(t.transforms):
            d = _inverse_distance(sub, d)
        return d
    raise TypeError(f"{type(t).__name__}.Inverse() is not a DistTransform")


def _dist_bound(m, d: float) -> float:
    """Metaball.MetaballDistBound (shapes.go:139, transform.go:339-341, :399-401)."""
    if isinstance(m, _TransformedMetaball):
        return _dist_bound(m.wrapped, _inverse_distance(m.transform, d))
    if isinstance(m, _VecScaleMetaball):
        return _dist_bound(m.wrapped, d * m.invMaxScale)
    _check_ball(m)
    return d


def ball_steps(m):
    """(forward MC_XF_* steps innermost first, primitive) of a metaball."""
    if isinstance(m, _TransformedMetaball):
        steps, prim = ball_steps(m.wrapped)
        return steps + m.transform._steps(), prim
    if isinstance(m, _VecScaleMetaball):
        steps, prim = ball_steps(m.wrapped)
        return steps + VecScale(m.scale)._steps(), prim
    if isinstance(m, _SDFMetaball):
        return [], m.sdf
    _check_ball(m)
    return [], m


class MetaballSolidT(Solid):
    """The CheckedFuncSolid that WeightedMetaballSolid returns
    (model3d/metaball.go:234-242)."""

    def __init__(self, f: MetaballFalloff, radiusThreshold: float, balls, weights, mn, mx):
        self.falloff, self.radiusThreshold = f, float(radiusThreshold)
        self.balls, self.weights = list(balls), [float(w) for w in weights]
        self.min, self.max = mn, mx

    def Min(self):
        return self.min

    def Max(self):
        return self.max


def WeightedMetaballSolid(f: Optional[MetaballFalloff], radiusThreshold: float,
                          balls: Sequence, weights: Sequence[float]) -> Solid:
    """model3d/metaball.go:165-242."""
    if len(balls) != len(weights):
        raise ValueError("number of balls must match number of weights")
    if f is None:
        f = QuarticMetaballFalloffFunc
    if not isinstance(f, (_InversePower, _Wyvill, _ExpFalloff)):
        raise NotLowerable("custom falloff functions have no device lowering")
    weights = [float(w) for w in weights]
    threshold = f(float(radiusThreshold))

    pos = [mb for mb, w in zip(balls, weights) if w > 0]
    if not pos:
        return NewRect(XYZ(0, 0, 0), XYZ(0, 0, 0))
    mn, mx = _ball_min(pos[0]), _ball_max(pos[0])
    for b in pos[1:]:
        mn = mn.Min(_ball_min(b))
        mx = mx.Max(_ball_max(b))
    for b in balls:
        _check_ball(b)

    def value_for_outset(x: float) -> float:
        s = 0.0
        for mb, w in zip(balls, weights):
            if w > 0:
                s += w * f(_dist_bound(mb, x))
        return s

    max_outset = mx.Dist(mn)
    min_outset = max_outset * 1e-8
    for _ in range(32):
        if value_for_outset(max_outset) > threshold:
            max_outset *= 2.0
        else:
            break
    if value_for_outset(max_outset) > threshold:
        raise ValueError("could not find maximum outset")
    for _ in range(32):
        mid = (min_outset + max_outset) / 2
        if value_for_outset(mid) > threshold:
            min_outset = mid
        else:
            max_outset = mid
    return MetaballSolidT(f, radiusThreshold, balls, weights,
                          mn.AddScalar(-max_outset), mx.AddScalar(max_outset))


def SignedMetaballSolid(f: Optional[MetaballFalloff], radiusThreshold: float,
                        pos: Sequence, neg: Sequence) -> Solid:
    """model3d/metaball.go:150-163."""
    balls = list(pos) + list(neg)
    return WeightedMetaballSolid(f, radiusThreshold, balls, [1.0] * len(pos) + [-1.0] * len(neg))


def MetaballSolid(f: Optional[MetaballFalloff], radiusThreshold: float, *m) -> Solid:
    """model3d/metaball.go:144-148."""
    return SignedMetaballSolid(f, radiusThreshold, m, [])
