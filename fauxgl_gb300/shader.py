"""Built-in shaders and textures of package fauxgl (shader.go, texture.go).

Only the three built-in shaders exist on the device. Their parameters are
copied into an fgc_shader struct at draw time; any other object assigned to
Context.Shader is rejected with UnsupportedShaderError (the reference would
run arbitrary Go code there; this implementation has no CPU fallback).
"""
import ctypes

import numpy as np

from . import _abi
from .geom import Color, Discard, Identity, Matrix, Vector


class UnsupportedShaderError(TypeError):
    """Context.Shader is not one of SolidColorShader, TextureShader, PhongShader."""


class ImageTexture:
    """ImageTexture (texture.go:21-31). texels: (H, W, 4) uint16 array of the
    alpha-premultiplied 16-bit RGBA values image.At(x, y).RGBA() returns."""

    def __init__(self, texels):
        t = np.ascontiguousarray(np.asarray(texels, dtype=np.uint16))
        assert t.ndim == 3 and t.shape[2] == 4
        self.texels = t
        self.Height, self.Width = int(t.shape[0]), int(t.shape[1])
        self._device = None

    @staticmethod
    def from_nrgba8(img):
        """Texture from an (H, W, 4) uint8 NRGBA image, converted the way
        color.NRGBA.RGBA() converts (16-bit, premultiplied by alpha)."""
        img = np.asarray(img, dtype=np.uint32)
        a = img[..., 3]
        out = np.empty(img.shape, dtype=np.uint16)
        for c in range(3):
            v = img[..., c] | (img[..., c] << 8)
            out[..., c] = (v * a // 0xff).astype(np.uint16)
        out[..., 3] = (a | (a << 8)).astype(np.uint16)
        return ImageTexture(out)


def NewImageTexture(texels):
    return ImageTexture(texels)


class SolidColorShader:
    """shader.go:10-27."""

    def __init__(self, matrix, color):
        self.Matrix = Matrix(matrix)
        self.Color = Color(*color)


class TextureShader:
    """shader.go:29-46."""

    def __init__(self, matrix, texture):
        self.Matrix = Matrix(matrix)
        self.Texture = texture


class PhongShader:
    """shader.go:48-96."""

    def __init__(self, matrix, light_direction, camera_position):
        self.Matrix = Matrix(matrix)
        self.LightDirection = Vector(*light_direction)
        self.CameraPosition = Vector(*camera_position)
        self.ObjectColor = Discard
        self.AmbientColor = Color(0.2, 0.2, 0.2, 1)
        self.DiffuseColor = Color(0.8, 0.8, 0.8, 1)
        self.SpecularColor = Color(1, 1, 1, 1)
        self.Texture = None
        self.SpecularPower = 32.0


def NewSolidColorShader(matrix, color):
    return SolidColorShader(matrix, color)


def NewTextureShader(matrix, texture):
    return TextureShader(matrix, texture)


def NewPhongShader(matrix, light_direction, camera_position):
    return PhongShader(matrix, light_direction, camera_position)


def to_fgc_shader(shader, texture_handle=None):
    """Copy a built-in shader's parameters into an fgc_shader struct.

    texture_handle is the device texture pointer (or None) the caller
    resolved for the shader's texture."""
    s = _abi.FgcShader()
    if type(shader) is SolidColorShader:
        s.kind = _abi.FGC_SHADER_SOLID_COLOR
        s.color[:] = list(shader.Color)
    elif type(shader) is TextureShader:
        s.kind = _abi.FGC_SHADER_TEXTURE
    elif type(shader) is PhongShader:
        s.kind = _abi.FGC_SHADER_PHONG
        s.color[:] = list(shader.ObjectColor)
        s.light_direction[:] = list(shader.LightDirection)
        s.camera_position[:] = list(shader.CameraPosition)
        s.ambient_color[:] = list(shader.AmbientColor)
        s.diffuse_color[:] = list(shader.DiffuseColor)
        s.specular_color[:] = list(shader.SpecularColor)
        s.specular_power = float(shader.SpecularPower)
    else:
        raise UnsupportedShaderError(
            "shader %r is not a built-in (SolidColorShader, TextureShader, PhongShader); "
            "custom shaders cannot run on the device" % (type(shader).__name__,))
    s.matrix[:] = list(shader.Matrix)
    s.texture = texture_handle
    return s


def shader_texture(shader):
    """The ImageTexture a shader samples, or None."""
    if type(shader) in (TextureShader, PhongShader):
        return shader.Texture
    return None
