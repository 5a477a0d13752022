"""Host-side value types of package fauxgl: Vector, VectorW, Color, Matrix.

These build scenes (camera matrices, light directions, colours) on the host,
exactly as the reference's Go code does; the device never recomputes them.
Every expression keeps the reference's left-to-right operation order so a
matrix built here has the bits the reference would build (Python floats are
IEEE binary64 with no fused multiply-add). Citations are fogleman/fauxgl
file:line.
"""
import math

MAX_FLOAT64 = 1.7976931348623157e308


def go_min(x, y):
    """math.Min: -Inf wins, then NaN, then -0 below +0."""
    if (math.isinf(x) and x < 0) or (math.isinf(y) and y < 0):
        return -math.inf
    if math.isnan(x) or math.isnan(y):
        return math.nan
    if x == 0 and x == y:
        return x if math.copysign(1.0, x) < 0 else y
    return x if x < y else y


def go_max(x, y):
    """math.Max: +Inf wins, then NaN, then +0 above -0."""
    if (math.isinf(x) and x > 0) or (math.isinf(y) and y > 0):
        return math.inf
    if math.isnan(x) or math.isnan(y):
        return math.nan
    if x == 0 and x == y:
        return y if math.copysign(1.0, x) < 0 else x
    return x if x > y else y


def Radians(degrees):
    """util.go:9-11."""
    return degrees * math.pi / 180


def Clamp(x, lo, hi):
    """util.go:74-82."""
    if x < lo:
        return lo
    if x > hi:
        return hi
    return x


class Vector(tuple):
    """Vector{X, Y, Z} (vector.go:8-10)."""
    __slots__ = ()

    def __new__(cls, x=0.0, y=0.0, z=0.0):
        return tuple.__new__(cls, (float(x), float(y), float(z)))

    X = property(lambda s: s[0])
    Y = property(lambda s: s[1])
    Z = property(lambda s: s[2])

    def Add(a, b):
        return Vector(a[0] + b[0], a[1] + b[1], a[2] + b[2])

    def Sub(a, b):
        return Vector(a[0] - b[0], a[1] - b[1], a[2] - b[2])

    def Mul(a, b):
        return Vector(a[0] * b[0], a[1] * b[1], a[2] * b[2])

    def Div(a, b):
        return Vector(a[0] / b[0], a[1] / b[1], a[2] / b[2])

    def MulScalar(a, s):
        return Vector(a[0] * s, a[1] * s, a[2] * s)

    def DivScalar(a, s):
        return Vector(a[0] / s, a[1] / s, a[2] / s)

    def Dot(a, b):
        return a[0] * b[0] + a[1] * b[1] + a[2] * b[2]

    def Cross(a, b):
        return Vector(a[1] * b[2] - a[2] * b[1], a[2] * b[0] - a[0] * b[2], a[0] * b[1] - a[1] * b[0])

    def Length(a):
        return math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])

    def Normalize(a):
        """vector.go:83-86: multiply by the reciprocal of the length."""
        r = 1 / math.sqrt(a[0] * a[0] + a[1] * a[1] + a[2] * a[2])
        return Vector(a[0] * r, a[1] * r, a[2] * r)

    def Negate(a):
        return Vector(-a[0], -a[1], -a[2])

    def Min(a, b):
        return Vector(go_min(a[0], b[0]), go_min(a[1], b[1]), go_min(a[2], b[2]))

    def Max(a, b):
        return Vector(go_max(a[0], b[0]), go_max(a[1], b[1]), go_max(a[2], b[2]))

    def MinComponent(a):
        return go_min(go_min(a[0], a[1]), a[2])

    def MaxComponent(a):
        return go_max(go_max(a[0], a[1]), a[2])

    def VectorW(a):
        return VectorW(a[0], a[1], a[2], 1.0)


def V(x, y, z):
    return Vector(x, y, z)


class VectorW(tuple):
    """VectorW{X, Y, Z, W} (vector.go:189-191)."""
    __slots__ = ()

    def __new__(cls, x=0.0, y=0.0, z=0.0, w=0.0):
        return tuple.__new__(cls, (float(x), float(y), float(z), float(w)))

    X = property(lambda s: s[0])
    Y = property(lambda s: s[1])
    Z = property(lambda s: s[2])
    W = property(lambda s: s[3])

    def Vector(a):
        return Vector(a[0], a[1], a[2])

    def Outside(a):
        x, y, z, w = a
        return x < -w or x > w or y < -w or y > w or z < -w or z > w


class Color(tuple):
    """Color{R, G, B, A} (color.go:17-19)."""
    __slots__ = ()

    def __new__(cls, r=0.0, g=0.0, b=0.0, a=0.0):
        return tuple.__new__(cls, (float(r), float(g), float(b), float(a)))

    R = property(lambda s: s[0])
    G = property(lambda s: s[1])
    B = property(lambda s: s[2])
    A = property(lambda s: s[3])

    def Alpha(c, alpha):
        return Color(c[0], c[1], c[2], alpha)

    def Add(a, b):
        return Color(a[0] + b[0], a[1] + b[1], a[2] + b[2], a[3] + b[3])

    def Mul(a, b):
        return Color(a[0] * b[0], a[1] * b[1], a[2] * b[2], a[3] * b[3])

    def MulScalar(a, s):
        return Color(a[0] * s, a[1] * s, a[2] * s, a[3] * s)

    def NRGBA(c):
        """color.go:56-63: clamp, scale by 255, truncate."""
        return tuple(int(Clamp(v, 0, 1) * 0xff) if not math.isnan(v) else 0 for v in c)


Discard = Color()
Transparent = Color()
Black = Color(0, 0, 0, 1)
White = Color(1, 1, 1, 1)


def Gray(x):
    return Color(x, x, x, 1)


def HexColor(x):
    """color.go:31-54 (3, 4, 6 or 8 hex digits, optional leading #)."""
    x = x.strip("#")
    r = g = b = 0
    a = 255
    if len(x) == 3:
        r, g, b = (int(c, 16) for c in x)
        r, g, b = (r << 4) | r, (g << 4) | g, (b << 4) | b
    elif len(x) == 4:
        r, g, b, a = (int(c, 16) for c in x)
        r, g, b, a = (r << 4) | r, (g << 4) | g, (b << 4) | b, (a << 4) | a
    elif len(x) == 6:
        r, g, b = int(x[0:2], 16), int(x[2:4], 16), int(x[4:6], 16)
    elif len(x) == 8:
        r, g, b, a = int(x[0:2], 16), int(x[2:4], 16), int(x[4:6], 16), int(x[6:8], 16)
    d = 0xff
    return Color(r / d, g / d, b / d, a / d)


def MakeColor(rgba16):
    """color.go:25-29 for a 16-bit premultiplied RGBA tuple."""
    d = 0xffff
    return Color(rgba16[0] / d, rgba16[1] / d, rgba16[2] / d, rgba16[3] / d)


class Matrix(tuple):
    """Row-major 4x4 FP64 matrix (matrix.go:5-10)."""
    __slots__ = ()

    def __new__(cls, *vals):
        if len(vals) == 1:
            vals = tuple(vals[0])
        assert len(vals) == 16
        return tuple.__new__(cls, tuple(float(v) for v in vals))

    def Mul(a, b):
        """matrix.go:188-207 (each entry summed left to right)."""
        m = [0.0] * 16
        for i in range(4):
            for j in range(4):
                m[4 * i + j] = (a[4 * i] * b[j] + a[4 * i + 1] * b[4 + j] + a[4 * i + 2] * b[8 + j]
                                + a[4 * i + 3] * b[12 + j])
        return Matrix(m)

    def MulPosition(a, b):
        """matrix.go:209-214."""
        return Vector(a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3],
                      a[4] * b[0] + a[5] * b[1] + a[6] * b[2] + a[7],
                      a[8] * b[0] + a[9] * b[1] + a[10] * b[2] + a[11])

    def MulPositionW(a, b):
        """matrix.go:216-222."""
        return VectorW(a[0] * b[0] + a[1] * b[1] + a[2] * b[2] + a[3],
                       a[4] * b[0] + a[5] * b[1] + a[6] * b[2] + a[7],
                       a[8] * b[0] + a[9] * b[1] + a[10] * b[2] + a[11],
                       a[12] * b[0] + a[13] * b[1] + a[14] * b[2] + a[15])

    def MulDirection(a, b):
        """matrix.go:224-229."""
        return Vector(a[0] * b[0] + a[1] * b[1] + a[2] * b[2],
                      a[4] * b[0] + a[5] * b[1] + a[6] * b[2],
                      a[8] * b[0] + a[9] * b[1] + a[10] * b[2]).Normalize()

    def Translate(m, v):
        return Translate(v).Mul(m)

    def Scale(m, v):
        return Scale(v).Mul(m)

    def Rotate(m, v, a):
        return Rotate(v, a).Mul(m)

    def Frustum(m, l, r, b, t, n, f):
        return Frustum(l, r, b, t, n, f).Mul(m)

    def Orthographic(m, l, r, b, t, n, f):
        return Orthographic(l, r, b, t, n, f).Mul(m)

    def Perspective(m, fovy, aspect, near, far):
        return Perspective(fovy, aspect, near, far).Mul(m)

    def LookAt(m, eye, center, up):
        return LookAt(eye, center, up).Mul(m)


def Identity():
    return Matrix(1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1, 0, 0, 0, 0, 1)


def Translate(v):
    return Matrix(1, 0, 0, v[0], 0, 1, 0, v[1], 0, 0, 1, v[2], 0, 0, 0, 1)


def Scale(v):
    return Matrix(v[0], 0, 0, 0, 0, v[1], 0, 0, 0, 0, v[2], 0, 0, 0, 0, 1)


def Rotate(v, a):
    """matrix.go:36-46."""
    v = Vector(*v).Normalize()
    s = math.sin(a)
    c = math.cos(a)
    m = 1 - c
    x, y, z = v
    return Matrix(m * x * x + c, m * x * y + z * s, m * z * x - y * s, 0,
                  m * x * y - z * s, m * y * y + c, m * y * z + x * s, 0,
                  m * z * x + y * s, m * y * z - x * s, m * z * z + c, 0,
                  0, 0, 0, 1)


def Frustum(l, r, b, t, n, f):
    """matrix.go:69-79."""
    t1 = 2 * n
    t2 = r - l
    t3 = t - b
    t4 = f - n
    return Matrix(t1 / t2, 0, (r + l) / t2, 0,
                  0, t1 / t3, (t + b) / t3, 0,
                  0, 0, (-f - n) / t4, (-t1 * f) / t4,
                  0, 0, -1, 0)


def Orthographic(l, r, b, t, n, f):
    """matrix.go:81-87."""
    return Matrix(2 / (r - l), 0, 0, -(r + l) / (r - l),
                  0, 2 / (t - b), 0, -(t + b) / (t - b),
                  0, 0, -2 / (f - n), -(f + n) / (f - n),
                  0, 0, 0, 1)


def Perspective(fovy, aspect, near, far):
    """matrix.go:89-93."""
    ymax = near * math.tan(fovy * math.pi / 360)
    xmax = ymax * aspect
    return Frustum(-xmax, xmax, -ymax, ymax, near, far)


def LookAt(eye, center, up):
    """matrix.go:95-105."""
    eye, center, up = Vector(*eye), Vector(*center), Vector(*up)
    z = eye.Sub(center).Normalize()
    x = up.Cross(z).Normalize()
    y = z.Cross(x)
    return Matrix(x[0], x[1], x[2], -x.Dot(eye),
                  y[0], y[1], y[2], -y.Dot(eye),
                  z[0], z[1], z[2], -z.Dot(eye),
                  0, 0, 0, 1)


def Screen(w, h):
    """matrix.go:119-128."""
    w2 = float(w) / 2
    h2 = float(h) / 2
    return Matrix(w2, 0, 0, w2, 0, -h2, 0, h2, 0, 0, 0.5, 0.5, 0, 0, 0, 1)
