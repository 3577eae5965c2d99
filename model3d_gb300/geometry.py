"""Coord3D and Matrix3 with model3d's float64 semantics.

Python floats are IEEE binary64 and every ``a * b + c`` is rounded after each
operation, which is the reference's behaviour on amd64 (Go does not fuse
there), so bounds computed here are bit-identical to the Go values.

References: model3d/coords.go:84-467, model3d/matrix.go:12-146.
"""
from __future__ import annotations

import math


def go_min(x: float, y: float) -> float:
    """math.Min: -Inf wins, then NaN, then -0 over +0."""
    if x == -math.inf or y == -math.inf:
        return -math.inf
    if x != x or y != y:
        return math.nan
    if x == 0 and y == 0:
        return x if math.copysign(1.0, x) < 0 else y
    return x if x < y else y


def go_max(x: float, y: float) -> float:
    """math.Max: +Inf wins, then NaN, then +0 over -0."""
    if x == math.inf or y == math.inf:
        return math.inf
    if x != x or y != y:
        return math.nan
    if x == 0 and y == 0:
        return y if math.copysign(1.0, x) < 0 else x
    return x if x > y else y


class Coord3D:
    """A 3-D coordinate (model3d/coords.go:84-89)."""

    __slots__ = ("X", "Y", "Z")

    def __init__(self, X: float = 0.0, Y: float = 0.0, Z: float = 0.0):
        self.X = float(X)
        self.Y = float(Y)
        self.Z = float(Z)

    def Array(self):
        return [self.X, self.Y, self.Z]

    def Add(self, c: "Coord3D") -> "Coord3D":
        return Coord3D(self.X + c.X, self.Y + c.Y, self.Z + c.Z)

    def Scale(self, s: float) -> "Coord3D":
        return Coord3D(self.X * s, self.Y * s, self.Z * s)

    def Sub(self, c: "Coord3D") -> "Coord3D":
        return self.Add(c.Scale(-1))

    def AddScalar(self, s: float) -> "Coord3D":
        return Coord3D(self.X + s, self.Y + s, self.Z + s)

    def Mul(self, c: "Coord3D") -> "Coord3D":
        return Coord3D(self.X * c.X, self.Y * c.Y, self.Z * c.Z)

    def Recip(self) -> "Coord3D":
        return Coord3D(1 / self.X, 1 / self.Y, 1 / self.Z)

    def Dot(self, c: "Coord3D") -> float:
        return self.X * c.X + self.Y * c.Y + self.Z * c.Z

    def Cross(self, c: "Coord3D") -> "Coord3D":
        return Coord3D(self.Y * c.Z - self.Z * c.Y, self.Z * c.X - self.X * c.Z,
                       self.X * c.Y - self.Y * c.X)

    def Norm(self) -> float:
        return math.sqrt(self.X * self.X + self.Y * self.Y + self.Z * self.Z)

    def Normalize(self) -> "Coord3D":
        return self.Scale(1 / self.Norm())

    def Mid(self, c: "Coord3D") -> "Coord3D":
        return self.Add(c).Scale(0.5)

    def Dist(self, c: "Coord3D") -> float:
        d1, d2, d3 = self.X - c.X, self.Y - c.Y, self.Z - c.Z
        return math.sqrt(d1 * d1 + d2 * d2 + d3 * d3)

    def Min(self, c: "Coord3D") -> "Coord3D":
        # A strict comparison decides math.Min; ties (+0/-0) and NaN go to go_min.
        a, b = self, c
        return Coord3D(a.X if a.X < b.X else (b.X if b.X < a.X else go_min(a.X, b.X)),
                       a.Y if a.Y < b.Y else (b.Y if b.Y < a.Y else go_min(a.Y, b.Y)),
                       a.Z if a.Z < b.Z else (b.Z if b.Z < a.Z else go_min(a.Z, b.Z)))

    def Max(self, c: "Coord3D") -> "Coord3D":
        a, b = self, c
        return Coord3D(a.X if a.X > b.X else (b.X if b.X > a.X else go_max(a.X, b.X)),
                       a.Y if a.Y > b.Y else (b.Y if b.Y > a.Y else go_max(a.Y, b.Y)),
                       a.Z if a.Z > b.Z else (b.Z if b.Z > a.Z else go_max(a.Z, b.Z)))

    def Sum(self) -> float:
        return self.X + self.Y + self.Z

    def Abs(self) -> "Coord3D":
        return Coord3D(abs(self.X), abs(self.Y), abs(self.Z))

    def MaxCoord(self) -> float:
        """model3d/coords.go:357-371 (NaN and ties follow its comparisons)."""
        if self.X > self.Y:
            return self.X if self.X > self.Z else self.Z
        return self.Y if self.Y > self.Z else self.Z

    def ProjectOut(self, c1: "Coord3D") -> "Coord3D":
        normed = c1.Normalize()
        return self.Sub(normed.Scale(normed.Dot(self)))

    def OrthoBasis(self):
        """model3d/coords.go:388-422."""
        absX, absY, absZ = abs(self.X), abs(self.Y), abs(self.Z)
        b1 = Coord3D()
        if absX > absY and absX > absZ:
            b1.X = self.Y / absX
            b1.Y = -self.X / absX
        else:
            b1.Y = self.Z
            b1.Z = -self.Y
            if absY > absZ:
                b1.Y /= absY
                b1.Z /= absY
            else:
                b1.Y /= absZ
                b1.Z /= absZ
        b2 = Coord3D(b1.Y * self.Z - b1.Z * self.Y, b1.Z * self.X - b1.X * self.Z,
                     b1.X * self.Y - b1.Y * self.X)
        return b1.Normalize(), b2.Normalize()

    def __eq__(self, o):  # Go ==: -0 == +0, NaN != NaN
        return isinstance(o, Coord3D) and self.X == o.X and self.Y == o.Y and self.Z == o.Z

    def __hash__(self):
        return hash((self.X + 0.0, self.Y + 0.0, self.Z + 0.0))

    def __repr__(self):
        return f"XYZ({self.X!r}, {self.Y!r}, {self.Z!r})"


def XYZ(x: float, y: float, z: float) -> Coord3D:
    return Coord3D(x, y, z)


def X(x: float) -> Coord3D:
    return Coord3D(x, 0, 0)


def Y(y: float) -> Coord3D:
    return Coord3D(0, y, 0)


def Z(z: float) -> Coord3D:
    return Coord3D(0, 0, z)


class Matrix3:
    """Row-major 3x3 matrix (model3d/matrix.go:12)."""

    __slots__ = ("m",)

    def __init__(self, m):
        self.m = [float(v) for v in m]
        if len(self.m) != 9:
            raise ValueError("Matrix3 needs 9 entries")

    def MulColumn(self, c: Coord3D) -> Coord3D:
        m = self.m
        return Coord3D(m[0] * c.X + m[1] * c.Y + m[2] * c.Z,
                       m[3] * c.X + m[4] * c.Y + m[5] * c.Z,
                       m[6] * c.X + m[7] * c.Y + m[8] * c.Z)

    def Mul(self, o: "Matrix3") -> "Matrix3":
        a, b = self.m, o.m
        return Matrix3([
            a[0] * b[0] + a[1] * b[3] + a[2] * b[6], a[0] * b[1] + a[1] * b[4] + a[2] * b[7],
            a[0] * b[2] + a[1] * b[5] + a[2] * b[8],
            a[3] * b[0] + a[4] * b[3] + a[5] * b[6], a[3] * b[1] + a[4] * b[4] + a[5] * b[7],
            a[3] * b[2] + a[4] * b[5] + a[5] * b[8],
            a[6] * b[0] + a[7] * b[3] + a[8] * b[6], a[6] * b[1] + a[7] * b[4] + a[8] * b[7],
            a[6] * b[2] + a[7] * b[5] + a[8] * b[8]])

    def Transpose(self) -> "Matrix3":
        m = self.m
        return Matrix3([m[0], m[3], m[6], m[1], m[4], m[7], m[2], m[5], m[8]])


def NewMatrix3Columns(c1: Coord3D, c2: Coord3D, c3: Coord3D) -> Matrix3:
    return Matrix3([c1.X, c2.X, c3.X, c1.Y, c2.Y, c3.Y, c1.Z, c2.Z, c3.Z])


def NewMatrix3Rotation(axis: Coord3D, angle: float) -> Matrix3:
    """model3d/matrix.go:25-40 (sin/cos from the host libm)."""
    x, y = axis.OrthoBasis()
    basis = NewMatrix3Columns(axis, x, y)
    c, s = math.cos(angle), math.sin(angle)
    rotation = Matrix3([1, 0, 0, 0, c, s, 0, -s, c])
    return basis.Mul(rotation).Mul(basis.Transpose())
