"""Reading and writing the reference's `.octrn` asset files (data only).

The reference loads its meshes and textures through a closed library (`octarine_mesh_read_from_file`,
`octarine_image_read_from_file`, source/main.c:526-559); only its headers are public
(source/external/octarine/octarine_mesh.h:21-25, octarine_image.h:78-87). The byte layout below
is the one the shipped assets have (checked against every file in the reference's assets folder):

    8 bytes   magic "eniratco"
    u32       kind: 1 mesh, 0 image
    u32       unused (written as 0)
    header    mesh:  OctarineMeshHeader {u32 size_of_data, u32 num_vertices, u32 num_indices}
              image: OctarineImageHeader {u64 size_of_data, u32 format, u16 width, height, depth,
                                          array_size, mip_levels, flags}
    data      mesh:  num_vertices x 32-byte vertices (position3, normal3, uv2: basic_vs's input,
                     basic_vs.c:3-7), then num_indices x u32
              image: size_of_data bytes of texels, rows tightly packed

All fields are little-endian. Image formats are OctarineImageFormat words: type in bits 0-3
(1 float, 2 unsigned float16, 3 unorm), bits per pixel in 4-11, channels in 12-15, flags above.
"""
import struct

import numpy as np

MAGIC = b"eniratco"
KIND_IMAGE, KIND_MESH = 0, 1
FORMAT_R8G8B8A8_UNORM = 0x4203
FORMAT_R16G16B16A16_FLOAT = 0x4401
FORMAT_R32G32B32A32_FLOAT = 0x4801
FORMAT_R8G8B8A8_UNORM_SRGB = 0x24203
_DTYPE = {FORMAT_R8G8B8A8_UNORM: (np.uint8, 4), FORMAT_R8G8B8A8_UNORM_SRGB: (np.uint8, 4),
          FORMAT_R16G16B16A16_FLOAT: (np.float16, 4), FORMAT_R32G32B32A32_FLOAT: (np.float32, 4)}
_MESH_HEADER = struct.Struct("<8sIIIII")      # magic, kind, unused, size, vertices, indices
_IMAGE_HEADER = struct.Struct("<8sIIQIHHHHHH")  # magic, kind, unused, size, format, w, h, d, array, mips, flags


class OctrnError(ValueError):
    pass


def _check_magic(magic, kind, want, path):
    if magic != MAGIC:
        raise OctrnError("%s: not an .octrn file" % path)
    if kind != want:
        raise OctrnError("%s: kind %d, expected %d" % (path, kind, want))


def read_mesh(path):
    """(vertices float32 (n, 8), indices uint32 (m,)) of a mesh file."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < _MESH_HEADER.size:
        raise OctrnError("%s: truncated header" % path)
    magic, kind, _, size, nv, ni = _MESH_HEADER.unpack_from(data)
    _check_magic(magic, kind, KIND_MESH, path)
    if size != nv * 32 + ni * 4 or len(data) < _MESH_HEADER.size + size:
        raise OctrnError("%s: %d vertices and %d indices do not fill %d data bytes" % (path, nv, ni, size))
    off = _MESH_HEADER.size
    vertices = np.frombuffer(data, np.float32, nv * 8, off).reshape(nv, 8).copy()
    indices = np.frombuffer(data, np.uint32, ni, off + nv * 32).copy()
    if ni and int(indices.max()) >= nv:
        raise OctrnError("%s: index out of range" % path)
    return vertices, indices


def write_mesh(path, vertices, indices):
    vertices = np.ascontiguousarray(vertices, np.float32).reshape(-1, 8)
    indices = np.ascontiguousarray(indices, np.uint32).ravel()
    size = vertices.nbytes + indices.nbytes
    with open(path, "wb") as f:
        f.write(_MESH_HEADER.pack(MAGIC, KIND_MESH, 0, size, len(vertices), len(indices)))
        f.write(vertices.tobytes())
        f.write(indices.tobytes())


def read_image(path):
    """(texels (height, width, channels), format word) of a single 2D image (no mips or arrays)."""
    with open(path, "rb") as f:
        data = f.read()
    if len(data) < _IMAGE_HEADER.size:
        raise OctrnError("%s: truncated header" % path)
    magic, kind, _, size, fmt, w, h, depth, array, mips, _flags = _IMAGE_HEADER.unpack_from(data)
    _check_magic(magic, kind, KIND_IMAGE, path)
    if fmt not in _DTYPE:
        raise OctrnError("%s: unsupported format 0x%x" % (path, fmt))
    if depth != 1 or array != 1 or mips != 1:
        raise OctrnError("%s: only single 2D images are supported" % path)
    dt, ch = _DTYPE[fmt]
    if size != w * h * ch * np.dtype(dt).itemsize or len(data) < _IMAGE_HEADER.size + size:
        raise OctrnError("%s: size does not match %dx%d" % (path, w, h))
    texels = np.frombuffer(data, dt, w * h * ch, _IMAGE_HEADER.size).reshape(h, w, ch).copy()
    return texels, fmt


def write_image(path, texels, fmt):
    dt, ch = _DTYPE[fmt]
    texels = np.ascontiguousarray(texels, dt)
    h, w = texels.shape[:2]
    if texels.size != w * h * ch:
        raise OctrnError("texels do not have %d channels" % ch)
    with open(path, "wb") as f:
        f.write(_IMAGE_HEADER.pack(MAGIC, KIND_IMAGE, 0, texels.nbytes, fmt, w, h, 1, 1, 1, 0))
        f.write(texels.tobytes())


def srgb_to_linear_rgba8(texels):
    """The reference's load-time conversion of an sRGB RGBA8 texture to linear (main.c:546-557):
    each channel decoded as byte * f32(1/255) (decode_u32_as_color, math.h:325-332), mapped by srgb_to_linear
    (math.h:386-395, evaluated in double and stored to f32) and re-encoded as (u32)(c * 255.f), a
    truncation (encode_color_as_u32, math.h:321-323) - alpha included, as the reference does."""
    v = texels.astype(np.float32) * np.float32(1.0 / 255.0)
    d = v.astype(np.float64)
    lin = np.where(d <= 0.04045, d / 12.92, ((d + 0.055) / 1.055) ** 2.4).astype(np.float32)
    return (lin * np.float32(255.0)).astype(np.uint32).astype(np.uint8)
