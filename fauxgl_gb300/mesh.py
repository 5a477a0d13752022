"""Mesh, Triangle, Line and Vertex of package fauxgl, stored as arrays.

The reference keeps a mesh as []*Triangle of 17-float64 Vertex values
(mesh.go:9-13, triangle.go:3-5, vertex.go:3-12). Here a mesh is a set of
per-corner float64 arrays (the triangle soup, no index sharing), which is what
the device takes: tri_pos (T,3,3), tri_nrm (T,3,3), tri_tex (T,3,2),
tri_col (T,3,4) and the same per line with 2 corners. BiUnitCube/FitInside and
Transform are restated on the host with the reference's operation order;
SmoothNormals[Threshold], SharpEdges and Silhouette run on the GPU
(meshops.DeviceMesh). smooth_normals_threshold_host / smooth_normals_host are
host restatements of the smoothing used to synthesise benchmark meshes where
the library is not loaded. Citations are fogleman/fauxgl file:line.
"""
import math

import numpy as np

from .geom import Identity, Matrix, Scale, Translate, Vector, go_max, go_min


def _normalize(v):
    """Vector.Normalize on (...,3) arrays (vector.go:83-86)."""
    x, y, z = v[..., 0], v[..., 1], v[..., 2]
    with np.errstate(divide="ignore", invalid="ignore"):  # zero vectors give NaN, as in Go
        r = 1 / np.sqrt(x * x + y * y + z * z)
        return np.stack([x * r, y * r, z * r], axis=-1)


def _cross(a, b):
    """Vector.Cross (vector.go:76-81)."""
    ax, ay, az = a[..., 0], a[..., 1], a[..., 2]
    bx, by, bz = b[..., 0], b[..., 1], b[..., 2]
    return np.stack([ay * bz - az * by, az * bx - ax * bz, ax * by - ay * bx], axis=-1)


def _dot(a, b):
    return a[..., 0] * b[..., 0] + a[..., 1] * b[..., 1] + a[..., 2] * b[..., 2]


def group_rows(rows):
    """Group id of each row of an (n, 3) float64 array: rows with equal bit
    patterns share an id (ids are 0..groups-1). The rows' 64-bit mixed hash is
    grouped first; the grouping is then checked row by row against each
    group's first row, and an exact sort of the rows replaces it if two
    different rows ever share a hash."""
    rows = np.ascontiguousarray(rows, dtype=np.float64)
    b = rows.view(np.uint64).reshape(-1, 3)

    def fmix(z):  # splitmix64 finaliser
        z = z ^ (z >> np.uint64(30))
        z = z * np.uint64(0xBF58476D1CE4E5B9)
        z = z ^ (z >> np.uint64(27))
        z = z * np.uint64(0x94D049BB133111EB)
        return z ^ (z >> np.uint64(31))

    with np.errstate(over="ignore"):
        h = fmix(b[:, 0] + np.uint64(0x9E3779B97F4A7C15))
        h = fmix(h ^ fmix(b[:, 1] + np.uint64(0x632BE59BD9B4E019)))
        h = fmix(h ^ fmix(b[:, 2] + np.uint64(0x2545F4914F6CDD1D)))
    _, first, inv = np.unique(h, return_index=True, return_inverse=True)
    inv = inv.ravel()
    if np.array_equal(b, b[first[inv]]):
        return inv
    keys = rows.view(np.dtype((np.void, 24))).ravel()
    _, inv = np.unique(keys, return_inverse=True)
    return inv.ravel()


def face_normals(tri_pos):
    """Triangle.Normal (triangle.go:33-37) for (T,3,3) positions."""
    e1 = tri_pos[:, 1] - tri_pos[:, 0]
    e2 = tri_pos[:, 2] - tri_pos[:, 0]
    return _normalize(_cross(e1, e2))


def mul_position(m, p):
    """Matrix.MulPosition (matrix.go:209-214) on (...,3) arrays."""
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    return np.stack([m[0] * x + m[1] * y + m[2] * z + m[3],
                     m[4] * x + m[5] * y + m[6] * z + m[7],
                     m[8] * x + m[9] * y + m[10] * z + m[11]], axis=-1)


def mul_direction(m, p):
    """Matrix.MulDirection (matrix.go:224-229) on (...,3) arrays."""
    x, y, z = p[..., 0], p[..., 1], p[..., 2]
    return _normalize(np.stack([m[0] * x + m[1] * y + m[2] * z,
                                m[4] * x + m[5] * y + m[6] * z,
                                m[8] * x + m[9] * y + m[10] * z], axis=-1))


class Vertex:
    """Vertex (vertex.go:3-12): Position, Normal, Texture, Color (Output is device-side)."""

    def __init__(self, Position=(0, 0, 0), Normal=(0, 0, 0), Texture=(0, 0, 0), Color=(0, 0, 0, 0)):
        self.Position = Vector(*Position)
        self.Normal = Vector(*Normal)
        self.Texture = Vector(*Texture)
        self.Color = tuple(float(c) for c in Color)


class Triangle:
    """Triangle{V1, V2, V3} (triangle.go:3-5)."""

    def __init__(self, V1, V2, V3):
        self.V1, self.V2, self.V3 = V1, V2, V3

    def FixNormals(self):
        """triangle.go:46-58."""
        p = np.array([self.V1.Position, self.V2.Position, self.V3.Position], dtype=np.float64)[None]
        n = Vector(*face_normals(p)[0])
        for v in (self.V1, self.V2, self.V3):
            if v.Normal == (0.0, 0.0, 0.0):
                v.Normal = n


def NewTriangle(v1, v2, v3):
    """triangle.go:7-11."""
    t = Triangle(v1, v2, v3)
    t.FixNormals()
    return t


def NewTriangleForPoints(p1, p2, p3):
    return NewTriangle(Vertex(p1), Vertex(p2), Vertex(p3))


class Line:
    """Line{V1, V2} (line.go:3-5)."""

    def __init__(self, V1, V2):
        self.V1, self.V2 = V1, V2


def NewLine(v1, v2):
    return Line(v1, v2)


def NewLineForPoints(p1, p2):
    return Line(Vertex(p1), Vertex(p2))


class Mesh:
    """Mesh{Triangles, Lines} (mesh.go:9-13) as per-corner arrays."""

    def __init__(self, tri_pos=None, tri_nrm=None, tri_tex=None, tri_col=None,
                 line_pos=None, line_nrm=None, line_tex=None, line_col=None):
        def arr(a, shape_tail):
            if a is None:
                return None
            a = np.ascontiguousarray(np.asarray(a, dtype=np.float64))
            return a.reshape((-1,) + shape_tail)

        self.tri_pos = arr(tri_pos, (3, 3))
        if self.tri_pos is None:
            self.tri_pos = np.zeros((0, 3, 3))
        self.tri_nrm = arr(tri_nrm, (3, 3))
        self.tri_tex = arr(tri_tex, (3, 2))
        self.tri_col = arr(tri_col, (3, 4))
        self.line_pos = arr(line_pos, (2, 3))
        if self.line_pos is None:
            self.line_pos = np.zeros((0, 2, 3))
        self.line_nrm = arr(line_nrm, (2, 3))
        self.line_tex = arr(line_tex, (2, 2))
        self.line_col = arr(line_col, (2, 4))
        self._device = None
        self._device_key = None
        self.resident = False

    # -- sizes ------------------------------------------------------------
    @property
    def ntri(self):
        return int(self.tri_pos.shape[0])

    @property
    def nline(self):
        return int(self.line_pos.shape[0])

    def dirty(self):
        """Forget the device copy after the arrays were changed in place."""
        self._device = None
        self._device_key = None

    def MakeResident(self):
        """Keep a device copy of this mesh between draws (no counterpart in
        package fauxgl, whose DrawMesh reads mesh.Triangles on every call).
        A draw of a mesh that is not resident uploads it for that draw only,
        so edits between draws are always seen; a resident mesh is uploaded
        once, and the methods here that change it drop the copy themselves,
        but an edit of its arrays in place must be followed by dirty()."""
        self.resident = True
        return self

    # -- construction from reference-style objects -------------------------
    @staticmethod
    def from_objects(triangles=(), lines=()):
        """NewMesh(triangles, lines) from Triangle / Line objects."""
        triangles = list(triangles)
        lines = list(lines)

        def gather(objs, names, attr, width):
            out = np.zeros((len(objs), len(names), width))
            for i, o in enumerate(objs):
                for c, n in enumerate(names):
                    v = getattr(getattr(o, n), attr)
                    out[i, c, :] = v[:width]
            return out

        tn = ("V1", "V2", "V3")
        ln = ("V1", "V2")
        return Mesh(gather(triangles, tn, "Position", 3), gather(triangles, tn, "Normal", 3),
                    gather(triangles, tn, "Texture", 2), gather(triangles, tn, "Color", 4),
                    gather(lines, ln, "Position", 3), gather(lines, ln, "Normal", 3),
                    gather(lines, ln, "Texture", 2), gather(lines, ln, "Color", 4))

    def Copy(self):
        c = lambda a: None if a is None else a.copy()
        return Mesh(c(self.tri_pos), c(self.tri_nrm), c(self.tri_tex), c(self.tri_col),
                    c(self.line_pos), c(self.line_nrm), c(self.line_tex), c(self.line_col))

    def Add(self, other):
        """mesh.go:49-53: append the other mesh's triangles and lines."""
        def cat(a, b, n_a, n_b, tail):
            if a is None and b is None:
                return None
            a = np.zeros((n_a,) + tail) if a is None else a
            b = np.zeros((n_b,) + tail) if b is None else b
            return np.concatenate([a, b])

        nt, no = self.ntri, other.ntri
        nl, nol = self.nline, other.nline
        self.tri_pos = np.concatenate([self.tri_pos, other.tri_pos])
        self.tri_nrm = cat(self.tri_nrm, other.tri_nrm, nt, no, (3, 3))
        self.tri_tex = cat(self.tri_tex, other.tri_tex, nt, no, (3, 2))
        self.tri_col = cat(self.tri_col, other.tri_col, nt, no, (3, 4))
        self.line_pos = np.concatenate([self.line_pos, other.line_pos])
        self.line_nrm = cat(self.line_nrm, other.line_nrm, nl, nol, (2, 3))
        self.line_tex = cat(self.line_tex, other.line_tex, nl, nol, (2, 2))
        self.line_col = cat(self.line_col, other.line_col, nl, nol, (2, 4))
        self.dirty()

    def SetColor(self, c):
        """mesh.go:55-59."""
        self.tri_col = np.empty((self.ntri, 3, 4))
        self.tri_col[:] = np.asarray(c, dtype=np.float64)
        self.dirty()

    # -- geometry -----------------------------------------------------------
    def BoundingBox(self):
        """mesh.go:153-165 (Box.Extend from EmptyBox, Min/Max per component)."""
        pts = [self.tri_pos.reshape(-1, 3), self.line_pos.reshape(-1, 3)]
        pts = np.concatenate(pts)
        if pts.shape[0] == 0:
            return Vector(), Vector()
        mn = [float(pts[0, k]) for k in range(3)]
        mx = list(mn)
        lo = pts.min(axis=0)
        hi = pts.max(axis=0)
        for k in range(3):
            mn[k] = go_min(mn[k], float(lo[k]))
            mx[k] = go_max(mx[k], float(hi[k]))
        return Vector(*mn), Vector(*mx)

    def Transform(self, matrix):
        """mesh.go:167-175 -> Triangle/Line.Transform (triangle.go:64-71, line.go:20-25)."""
        m = tuple(matrix)
        self.tri_pos = mul_position(m, self.tri_pos)
        if self.tri_nrm is not None:
            self.tri_nrm = mul_direction(m, self.tri_nrm)
        else:
            self.tri_nrm = mul_direction(m, np.zeros_like(self.tri_pos))
        self.line_pos = mul_position(m, self.line_pos)
        if self.line_nrm is not None:
            self.line_nrm = mul_direction(m, self.line_nrm)
        else:
            self.line_nrm = mul_direction(m, np.zeros_like(self.line_pos))
        self.dirty()

    def FitInside(self, box_min, box_max, anchor):
        """mesh.go:142-151."""
        bmin, bmax = Vector(*box_min), Vector(*box_max)
        mn, mx = self.BoundingBox()
        box_size = bmax.Sub(bmin)
        size = mx.Sub(mn)
        scale = box_size.Div(size).MinComponent()
        extra = box_size.Sub(size.MulScalar(scale))
        matrix = Identity()
        matrix = matrix.Translate(mn.Negate())
        matrix = matrix.Scale(Vector(scale, scale, scale))
        matrix = matrix.Translate(bmin.Add(extra.Mul(Vector(*anchor))))
        self.Transform(matrix)
        return matrix

    def BiUnitCube(self):
        """mesh.go:127-130."""
        return self.FitInside((-1, -1, -1), (1, 1, 1), (0.5, 0.5, 0.5))

    def UnitCube(self):
        """mesh.go:122-125."""
        return self.FitInside((-0.5, -0.5, -0.5), (0.5, 0.5, 0.5), (0.5, 0.5, 0.5))

    # -- on the GPU (meshops.DeviceMesh): upload, operate, read back ------------
    def SmoothNormalsThreshold(self, radians):
        """mesh.go:80-103 on the GPU: each corner's normal becomes the normalised
        sum, in corner order, of the normals at the same position whose dot
        product with it is at least cos(radians)."""
        from .meshops import DeviceMesh
        d = DeviceMesh.upload(Mesh(self.tri_pos, self.tri_nrm if self.tri_nrm is not None
                                   else np.zeros_like(self.tri_pos)))
        d.SmoothNormalsThreshold(radians)
        self.tri_nrm = d.download().tri_nrm
        self.dirty()

    def SmoothNormals(self):
        """mesh.go:105-120 on the GPU: per position, the normalised sum of all its normals."""
        from .meshops import DeviceMesh
        d = DeviceMesh.upload(Mesh(self.tri_pos, self.tri_nrm if self.tri_nrm is not None
                                   else np.zeros_like(self.tri_pos)))
        d.SmoothNormals()
        self.tri_nrm = d.download().tri_nrm
        self.dirty()

    def SharpEdges(self, angle_threshold):
        """mesh.go:258-292 on the GPU: a line Mesh of the edges whose two faces
        meet at more than angle_threshold radians."""
        from .meshops import DeviceMesh
        return DeviceMesh.upload(Mesh(self.tri_pos)).SharpEdges(angle_threshold).download()

    def Silhouette(self, eye, offset):
        """mesh.go:207-209 / silhouette.go:3-53 on the GPU: a line Mesh."""
        from .meshops import DeviceMesh
        src = Mesh(self.tri_pos, self.tri_nrm if self.tri_nrm is not None else np.zeros_like(self.tri_pos))
        return DeviceMesh.upload(src).Silhouette(eye, offset).download()


def _position_groups(mesh):
    """Group corners by Position as Go's map[Vector] does (== on float64,
    so -0 and +0 are one key; a NaN position is never found). Returns (inv,
    order, starts, counts, nan) where order lists corner indices grouped by
    key, each group in corner (triangle, then V1..V3) order."""
    p = mesh.tri_pos.reshape(-1, 3) + 0.0  # -0 -> +0
    nan = np.isnan(p).any(axis=1)
    inv = group_rows(p)
    order = np.argsort(inv, kind="stable")
    counts = np.bincount(inv)
    starts = np.concatenate([[0], np.cumsum(counts)[:-1]])
    return inv, order, starts, counts, nan


def smooth_normals_threshold_host(mesh, radians):
    """Host restatement of SmoothNormalsThreshold (mesh.go:80-103), for
    synthesising meshes without the library: the same bits as the GPU's."""
    threshold = math.cos(radians)
    nrm = (mesh.tri_nrm if mesh.tri_nrm is not None else np.zeros_like(mesh.tri_pos)).reshape(-1, 3)
    inv, order, starts, counts, nan = _position_groups(mesh)
    gmax = int(counts.max()) if counts.size else 0
    member = np.full((counts.size, gmax), -1, dtype=np.int64)
    rank = np.arange(order.size) - np.repeat(starts, counts)
    member[inv[order], rank] = order
    acc = np.zeros_like(nrm)
    mine = nrm
    for k in range(gmax):
        idx = member[inv, k]
        valid = idx >= 0
        x = nrm[np.where(valid, idx, 0)]
        take = valid & (_dot(x, mine) >= threshold)
        # adding +0 for a skipped normal leaves the running sum unchanged:
        # the sum starts at +0 and is never -0
        acc = acc + np.where(take[:, None], x, 0.0)
    acc[nan] = 0.0  # a NaN key finds no normals: the zero vector (normalises to NaN)
    mesh.tri_nrm = _normalize(acc).reshape(-1, 3, 3)
    mesh.dirty()


def smooth_normals_host(mesh):
    """Host restatement of SmoothNormals (mesh.go:105-120)."""
    nrm = (mesh.tri_nrm if mesh.tri_nrm is not None else np.zeros_like(mesh.tri_pos)).reshape(-1, 3)
    inv, order, starts, counts, nan = _position_groups(mesh)
    sums = np.zeros((counts.size, 3))
    gmax = int(counts.max()) if counts.size else 0
    member = np.full((counts.size, gmax), -1, dtype=np.int64)
    rank = np.arange(order.size) - np.repeat(starts, counts)
    member[inv[order], rank] = order
    for k in range(gmax):
        idx = member[:, k]
        valid = idx >= 0
        sums = sums + np.where(valid[:, None], nrm[np.where(valid, idx, 0)], 0.0)
    out = _normalize(sums)[inv]
    out[nan] = 0.0  # a NaN key's lookup finds nothing: the zero Vector
    mesh.tri_nrm = out.reshape(-1, 3, 3)
    mesh.dirty()


def NewTriangleMesh(tri_pos, tri_nrm=None, tri_tex=None, tri_col=None):
    return Mesh(tri_pos, tri_nrm, tri_tex, tri_col)


def NewLineMesh(line_pos, line_nrm=None, line_tex=None, line_col=None):
    return Mesh(None, None, None, None, line_pos, line_nrm, line_tex, line_col)


def NewEmptyMesh():
    return Mesh()
