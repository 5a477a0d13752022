"""fauxgl_gb300: FauxGL's triangle pipeline on GB300 (sm_103a).

The public names mirror package fauxgl (fogleman/fauxgl) so programs read the
same: NewContext, Context.DrawMesh / DrawTriangles / DrawLines,
ClearColorBuffer[With], ClearDepthBuffer[With], the Cull / FrontFace /
DepthBias / AlphaBlend / Wireframe / ReadDepth / WriteDepth / WriteColor
fields, and the built-in SolidColorShader, TextureShader and PhongShader.
Drawing runs only in libfauxglcuda's CUDA kernels; see context.py.
"""
from .geom import (MAX_FLOAT64, Black, Clamp, Color, Discard, Frustum, Gray, HexColor, Identity, LookAt,
                   MakeColor, Matrix, Orthographic, Perspective, Radians, Rotate, Scale, Screen, Translate,
                   Transparent, V, Vector, VectorW, White)
from .mesh import (Line, Mesh, NewEmptyMesh, NewLine, NewLineForPoints, NewLineMesh, NewTriangle,
                   NewTriangleForPoints, NewTriangleMesh, Triangle, Vertex)
from .shapes import NewCone, NewCube, NewCylinder, NewIcosahedron, NewPlane, NewSphere
from .shader import (ImageTexture, NewImageTexture, NewPhongShader, NewSolidColorShader, NewTextureShader,
                     PhongShader, SolidColorShader, TextureShader, UnsupportedShaderError)

__all__ = [n for n in dir() if not n.startswith("_")]


def __getattr__(name):
    # The context layer needs the CUDA library; import it lazily so the host
    # helpers (scenes, meshes, matrices) are usable where it is not built.
    if name in ("Context", "NewContext", "RasterizeInfo", "FaceCW", "FaceCCW", "CullNone", "CullFront",
                "CullBack", "PRECISION_PLAIN", "PRECISION_MIXED"):
        from . import context
        return getattr(context, name)
    if name in ("LoadSTL", "DeviceMesh"):
        from . import meshops
        return getattr(meshops, name)
    raise AttributeError(name)
