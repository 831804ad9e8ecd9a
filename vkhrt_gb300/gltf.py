"""glTF 2.0 ingest for hair models: stands in for the reference's assimp loader
(ModelLoader::LoadFromFile, source/resources/model/model_loader.cpp:274-336; ProcessMesh :139-206;
ProcessNodes and Node::GetWorldMatrix, model.cpp:6-18).

Reads `.gltf` (JSON with external or base64 `data:` buffers) and `.glb` (binary container).
Every mesh primitive drawn by a node becomes one `Primitive`:

* LINES (mode 1) and LINE_STRIP (mode 3) -> hair: vertex positions and line index pairs, the
  input `GenerateLines` (geometry_processor.cpp:45-67) consumes; a strip of n vertices gives the
  n - 1 pairs (i, i + 1), as assimp's line faces do. An optional per-vertex scalar attribute
  `_RADIUS` (an application attribute; glTF has no standard hair radius) gives radii, otherwise
  the BLAS's constant radius applies.
* TRIANGLES (mode 4, default) -> a triangle mesh with its NORMAL attribute when present, and its
  material's albedo as the reference's loader reads it (model_loader.cpp:58-120): the base colour
  factor, and the base colour texture sampled at its TEXCOORD_n. Texels are the image's 8-bit
  values / 255, unconverted (the reference uploads them as R8G8B8A8_UNORM, model_loader.cpp:38).
  PNG images (8-bit, not interlaced) are decoded here; other image formats leave the map out and
  say so in `Primitive.note`.

Each primitive carries the world matrix of its node (the product of the node path's matrices or
TRS, column-vector convention, as glTF defines), which becomes the BLAS transform.
"""
from __future__ import annotations

import base64
import zlib
import json
import os
import struct
from dataclasses import dataclass

import numpy as np

_COMPONENT = {5120: np.int8, 5121: np.uint8, 5122: np.int16, 5123: np.uint16, 5125: np.uint32, 5126: np.float32}
_NCOMP = {"SCALAR": 1, "VEC2": 2, "VEC3": 3, "VEC4": 4, "MAT4": 16}
LINES, LINE_STRIP, TRIANGLES = 1, 3, 4


@dataclass
class Primitive:
    kind: str                          # "lines" or "triangles"
    vertices: np.ndarray               # (nv, 3) float32
    indices: np.ndarray                # (n, 2) line pairs or (n, 3) triangles, uint32
    transform: np.ndarray              # (4, 4) float32 row-major object -> world
    radius: np.ndarray | None = None   # (nv,) float32 (lines, from _RADIUS)
    normals: np.ndarray | None = None  # (nv, 3) float32 (triangles, from NORMAL)
    name: str = ""
    texcoords: np.ndarray | None = None    # (nv, 2) float32 (triangles with a base colour texture)
    albedo_factor: tuple = (1.0, 1.0, 1.0, 1.0)
    albedo_map: np.ndarray | None = None   # (h, w, 4) float32, row 0 at v = 0
    note: str = ""                         # why a texture was left out

    def blas_input(self, hair_type=None, **kw):
        """BLASInput for this primitive: lines as `hair_type` (BLASType.ePhantom, eLSS or eDOTS),
        triangles as BLASType.eMesh. Extra keyword arguments go to BLASInput."""
        from . import BLASInput, BLASType
        if self.kind == "triangles":
            return BLASInput(type=BLASType.eMesh, vertices=self.vertices, tri_indices=self.indices,
                             normals=self.normals, transform=self.transform, texcoords=self.texcoords,
                             albedo_factor=self.albedo_factor, albedo_map=self.albedo_map, **kw)
        return BLASInput(type=BLASType(hair_type if hair_type is not None else BLASType.ePhantom),
                         vertices=self.vertices, radius=self.radius, line_indices=self.indices,
                         transform=self.transform, **kw)


class GltfError(ValueError):
    pass


def _read_container(path: str) -> tuple[dict, bytes | None]:
    with open(path, "rb") as f:
        data = f.read()
    if data[:4] != b"glTF":
        return json.loads(data.decode("utf-8")), None
    if len(data) < 20:
        raise GltfError(f"{path}: truncated GLB header")
    magic, version, length = struct.unpack_from("<4sII", data, 0)
    if version != 2:
        raise GltfError(f"{path}: GLB version {version}, only 2 is supported")
    off, doc, binchunk = 12, None, None
    while off + 8 <= min(length, len(data)):
        clen, ctype = struct.unpack_from("<II", data, off)
        chunk = data[off + 8:off + 8 + clen]
        if ctype == 0x4E4F534A:  # JSON
            doc = json.loads(chunk.decode("utf-8"))
        elif ctype == 0x004E4942 and binchunk is None:  # BIN
            binchunk = chunk
        off += 8 + clen
    if doc is None:
        raise GltfError(f"{path}: GLB without a JSON chunk")
    return doc, binchunk


def _buffers(doc: dict, base_dir: str, glb_bin: bytes | None) -> list[bytes]:
    out = []
    for i, b in enumerate(doc.get("buffers", [])):
        uri = b.get("uri")
        if uri is None:
            if glb_bin is None:
                raise GltfError(f"buffer {i} has no uri and there is no GLB binary chunk")
            out.append(glb_bin)
        elif uri.startswith("data:"):
            out.append(base64.b64decode(uri.split(",", 1)[1]))
        else:
            with open(os.path.join(base_dir, uri), "rb") as f:
                out.append(f.read())
    return out


def _accessor(doc: dict, bufs: list[bytes], index: int) -> np.ndarray:
    acc = doc["accessors"][index]
    dt = np.dtype(_COMPONENT[acc["componentType"]])
    nc = _NCOMP[acc["type"]]
    count = acc["count"]
    if "bufferView" not in acc:  # all zeros (sparse accessors are not supported)
        return np.zeros((count, nc) if nc > 1 else count, dt)
    if "sparse" in acc:
        raise GltfError("sparse accessors are not supported")
    view = doc["bufferViews"][acc["bufferView"]]
    raw = bufs[view["buffer"]]
    start = view.get("byteOffset", 0) + acc.get("byteOffset", 0)
    elem = dt.itemsize * nc
    stride = view.get("byteStride", elem) or elem
    if stride == elem:
        arr = np.frombuffer(raw, dt, count * nc, start)
    else:
        rows = np.frombuffer(raw, np.uint8, (count - 1) * stride + elem, start).copy() if count else np.zeros(0, np.uint8)
        arr = np.lib.stride_tricks.as_strided(rows, (count, elem), (stride, 1)).copy().view(dt).reshape(-1)
    arr = arr.reshape(count, nc) if nc > 1 else arr.reshape(count)
    return np.array(arr)


def _node_matrix(node: dict) -> np.ndarray:
    if "matrix" in node:
        return np.asarray(node["matrix"], np.float64).reshape(4, 4).T  # stored column major
    t = np.asarray(node.get("translation", [0, 0, 0]), np.float64)
    x, y, z, w = node.get("rotation", [0, 0, 0, 1])
    s = np.asarray(node.get("scale", [1, 1, 1]), np.float64)
    r = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                  [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                  [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
    m = np.eye(4)
    m[:3, :3] = r * s[None, :]
    m[:3, 3] = t
    return m


def decode_png(data: bytes) -> np.ndarray:
    """An 8-bit, non-interlaced PNG (grey, grey + alpha, RGB or RGBA) as (h, w, 4) float32 texels
    = byte / 255, alpha 1 where the image has none. Unfilters the five PNG row filters (None, Sub,
    Up, Average, Paeth) as the PNG specification defines them."""
    if data[:8] != b"\x89PNG\r\n\x1a\n":
        raise GltfError("not a PNG image")
    off, idat, hdr = 8, [], None
    while off + 8 <= len(data):
        n, kind = struct.unpack_from(">I4s", data, off)
        body = data[off + 8:off + 8 + n]
        if kind == b"IHDR":
            hdr = struct.unpack(">IIBBBBB", body)
        elif kind == b"IDAT":
            idat.append(body)
        elif kind == b"IEND":
            break
        off += 12 + n
    if hdr is None:
        raise GltfError("PNG without IHDR")
    w, h, depth, ctype, _, _, interlace = hdr
    channels = {0: 1, 2: 3, 4: 2, 6: 4}.get(ctype)
    if depth != 8 or channels is None or interlace:
        raise GltfError(f"PNG of bit depth {depth}, colour type {ctype}, interlace {interlace} is not supported")
    raw = zlib.decompress(b"".join(idat))
    stride = w * channels
    if len(raw) != h * (stride + 1):
        raise GltfError("PNG data size does not match its header")
    img = np.zeros((h, stride), np.int32)
    prev = np.zeros(stride, np.int32)
    for y in range(h):
        f = raw[y * (stride + 1)]
        row = np.frombuffer(raw, np.uint8, stride, y * (stride + 1) + 1).astype(np.int32)
        if f == 0:
            cur = row
        elif f == 1:  # Sub: a running sum per channel
            cur = np.cumsum(row.reshape(w, channels), axis=0).reshape(-1) & 255
        elif f == 2:
            cur = (row + prev) & 255
        elif f in (3, 4):  # these depend on the reconstructed byte to the left
            cur = np.zeros(stride, np.int32)
            for x in range(stride):
                a = int(cur[x - channels]) if x >= channels else 0
                b = int(prev[x])
                c = int(prev[x - channels]) if x >= channels else 0
                if f == 3:
                    pred = (a + b) >> 1
                else:
                    pa, pb, pc = abs(b - c), abs(a - c), abs(a + b - 2 * c)
                    pred = a if pa <= pb and pa <= pc else (b if pb <= pc else c)
                cur[x] = (int(row[x]) + pred) & 255
        else:
            raise GltfError(f"PNG row filter {f}")
        img[y] = cur
        prev = cur
    px = img.reshape(h, w, channels).astype(np.float32) / np.float32(255.0)
    out = np.ones((h, w, 4), np.float32)
    if channels in (1, 2):
        out[..., :3] = px[..., :1]
        if channels == 2:
            out[..., 3] = px[..., 1]
    else:
        out[..., :channels] = px
    return out


def load(path: str) -> list[Primitive]:
    """The primitives of the default scene (or of every root node), in node order."""
    doc, glb_bin = _read_container(path)
    base_dir = os.path.dirname(os.path.abspath(path))
    bufs = _buffers(doc, base_dir, glb_bin)
    nodes = doc.get("nodes", [])
    scenes = doc.get("scenes", [])
    if scenes:
        roots = scenes[doc.get("scene", 0)].get("nodes", [])
    else:
        children = {c for n in nodes for c in n.get("children", [])}
        roots = [i for i in range(len(nodes)) if i not in children]
    out: list[Primitive] = []
    stack = [(r, np.eye(4)) for r in reversed(roots)]
    guard = 0
    while stack:
        guard += 1
        if guard > 1_000_000:
            raise GltfError("node graph too deep or cyclic")
        ni, parent = stack.pop()
        node = nodes[ni]
        world = parent @ _node_matrix(node)
        if "mesh" in node:
            mesh = doc["meshes"][node["mesh"]]
            for pi, prim in enumerate(mesh.get("primitives", [])):
                out.extend(_primitive(doc, bufs, prim, world, f"{mesh.get('name', node.get('name', ''))}:{pi}",
                                      base_dir))
        for c in reversed(node.get("children", [])):
            stack.append((c, world))
    return out


def _image(doc, bufs, base_dir, index) -> tuple[bytes, str]:
    """An image's bytes and MIME type (from a file, a data URI or a buffer view)."""
    im = doc["images"][index]
    if "bufferView" in im:
        view = doc["bufferViews"][im["bufferView"]]
        start = view.get("byteOffset", 0)
        return bufs[view["buffer"]][start:start + view["byteLength"]], im.get("mimeType", "")
    uri = im.get("uri", "")
    if uri.startswith("data:"):
        head, body = uri.split(",", 1)
        return base64.b64decode(body), head[5:].split(";")[0]
    with open(os.path.join(base_dir, uri), "rb") as f:
        data = f.read()
    return data, "image/png" if uri.lower().endswith(".png") else ""


def _material(doc, bufs, base_dir, prim, attrs, nverts):
    """(albedo factor, texcoords, albedo map, note) of a triangle primitive's material."""
    if "material" not in prim:
        return (1.0, 1.0, 1.0, 1.0), None, None, ""
    pbr = doc["materials"][prim["material"]].get("pbrMetallicRoughness", {})
    factor = tuple(float(x) for x in pbr.get("baseColorFactor", [1.0, 1.0, 1.0, 1.0]))
    tex = pbr.get("baseColorTexture")
    if tex is None:
        return factor, None, None, ""
    key = f"TEXCOORD_{tex.get('texCoord', 0)}"
    if key not in attrs:
        return factor, None, None, f"base colour texture without {key}"
    acc = doc["accessors"][attrs[key]]
    tc = _accessor(doc, bufs, attrs[key]).astype(np.float32).reshape(-1, 2)
    if acc.get("normalized"):  # unsigned byte / short texture coordinates
        tc /= np.float32(np.iinfo(_COMPONENT[acc["componentType"]]).max)
    if len(tc) != nverts:
        raise GltfError(f"{key} has {len(tc)} entries for {nverts} vertices")
    source = doc["textures"][tex["index"]].get("source")
    if source is None:
        return factor, None, None, "texture without an image source"
    data, mime = _image(doc, bufs, base_dir, source)
    if mime != "image/png" and data[:8] != b"\x89PNG\r\n\x1a\n":
        return factor, None, None, f"image {source} ({mime or 'unknown type'}) is not a PNG: map left out"
    return factor, np.ascontiguousarray(tc), decode_png(data), ""


def _primitive(doc, bufs, prim, world, name, base_dir="") -> list[Primitive]:
    mode = prim.get("mode", TRIANGLES)
    attrs = prim.get("attributes", {})
    if "POSITION" not in attrs:
        raise GltfError(f"{name}: primitive without POSITION")
    v = np.ascontiguousarray(_accessor(doc, bufs, attrs["POSITION"]), np.float32).reshape(-1, 3)
    idx = (np.asarray(_accessor(doc, bufs, prim["indices"]), np.uint32).reshape(-1) if "indices" in prim
           else np.arange(len(v), dtype=np.uint32))
    xf = world.astype(np.float32)
    if mode == LINES:
        pairs = idx[: len(idx) // 2 * 2].reshape(-1, 2)
    elif mode == LINE_STRIP:
        pairs = np.stack([idx[:-1], idx[1:]], axis=1) if len(idx) >= 2 else np.zeros((0, 2), np.uint32)
    elif mode == TRIANGLES:
        nrm = (np.ascontiguousarray(_accessor(doc, bufs, attrs["NORMAL"]), np.float32).reshape(-1, 3)
               if "NORMAL" in attrs else None)
        factor, tc, amap, note = _material(doc, bufs, base_dir, prim, attrs, len(v))
        return [Primitive("triangles", v, idx[: len(idx) // 3 * 3].reshape(-1, 3), xf, normals=nrm, name=name,
                          texcoords=tc, albedo_factor=factor, albedo_map=amap, note=note)]
    else:
        return []  # points, line loops, strips and fans of triangles are not hair or meshes here
    rad = (np.ascontiguousarray(_accessor(doc, bufs, attrs["_RADIUS"]), np.float32).reshape(-1)
           if "_RADIUS" in attrs else None)
    return [Primitive("lines", v, np.ascontiguousarray(pairs, np.uint32), xf, radius=rad, name=name)]
