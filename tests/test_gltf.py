"""glTF ingest (vkhrt_gb300.gltf): hair lines and triangle meshes, external buffers, data URIs,
GLB containers, interleaved accessors and node transforms. The files are written here."""
import base64
import json
import struct

import numpy as np
import pytest

import vkhrt_gb300 as H
from vkhrt_gb300 import gltf


def _doc_and_blob(strip: bool, interleave: bool):
    """Two strands (a LINE_STRIP primitive each, or one LINES primitive with index pairs), a
    quad mesh with normals, and a node tree: root (translation) -> hair node (rotation + scale),
    root -> mesh node (matrix)."""
    rng = np.random.default_rng(3)
    sv = rng.normal(size=(10, 3)).astype(np.float32)  # strand vertices, 5 per strand
    rad = np.linspace(0.004, 0.001, 10).astype(np.float32)
    mv = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    mn = np.tile(np.array([[0, 0, 1]], np.float32), (4, 1))
    tri = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    blob = bytearray()
    views, accs = [], []

    def add(arr, target=None, stride=None):
        while len(blob) % 4:
            blob.append(0)
        views.append({"buffer": 0, "byteOffset": len(blob), "byteLength": arr.nbytes, **({"byteStride": stride} if stride else {})})
        blob.extend(arr.tobytes())
        return len(views) - 1

    def acc(view, ctype, count, typ, off=0):
        accs.append({"bufferView": view, "componentType": ctype, "count": count, "type": typ, "byteOffset": off})
        return len(accs) - 1

    a_sv = acc(add(sv), 5126, 10, "VEC3")
    a_rad = acc(add(rad), 5126, 10, "SCALAR")
    if interleave:  # position and normal interleaved, 24-byte stride
        inter = np.concatenate([mv, mn], axis=1).astype(np.float32)
        vi = add(inter, stride=24)
        a_mv, a_mn = acc(vi, 5126, 4, "VEC3", 0), acc(vi, 5126, 4, "VEC3", 12)
    else:
        a_mv, a_mn = acc(add(mv), 5126, 4, "VEC3"), acc(add(mn), 5126, 4, "VEC3")
    a_tri = acc(add(tri), 5123, 6, "SCALAR")
    if strip:
        s0 = acc(add(np.arange(0, 5, dtype=np.uint32)), 5125, 5, "SCALAR")
        s1 = acc(add(np.arange(5, 10, dtype=np.uint32)), 5125, 5, "SCALAR")
        hair_prims = [{"attributes": {"POSITION": a_sv, "_RADIUS": a_rad}, "indices": s, "mode": 3} for s in (s0, s1)]
        pairs = [np.stack([np.arange(b, b + 4), np.arange(b + 1, b + 5)], 1) for b in (0, 5)]
    else:
        pr = np.concatenate([np.stack([np.arange(b, b + 4), np.arange(b + 1, b + 5)], 1) for b in (0, 5)]).astype(np.uint32)
        li = acc(add(pr.reshape(-1)), 5125, pr.size, "SCALAR")
        hair_prims = [{"attributes": {"POSITION": a_sv, "_RADIUS": a_rad}, "indices": li, "mode": 1}]
        pairs = [pr]
    c, s_ = np.cos(0.3), np.sin(0.3)
    rot = [0.0, np.sin(0.15), 0.0, np.cos(0.15)]  # 0.3 rad about +y
    mesh_m = np.eye(4)
    mesh_m[:3, 3] = [0.5, -0.2, 0.1]
    doc = {
        "asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0]}],
        "nodes": [{"translation": [0.0, 1.0, 0.0], "children": [1, 2]},
                  {"mesh": 0, "rotation": rot, "scale": [2.0, 2.0, 2.0]},
                  {"mesh": 1, "matrix": mesh_m.T.reshape(-1).tolist()}],
        "meshes": [{"name": "hair", "primitives": hair_prims},
                   {"name": "tie", "primitives": [{"attributes": {"POSITION": a_mv, "NORMAL": a_mn}, "indices": a_tri}]}],
        "accessors": accs, "bufferViews": views,
        "buffers": [{"byteLength": len(blob)}],
    }
    root = np.eye(4)
    root[1, 3] = 1.0
    hair_w = root.copy()
    rs = np.array([[c, 0, s_], [0, 1, 0], [-s_, 0, c]]) * 2.0
    hm = np.eye(4)
    hm[:3, :3] = rs
    hair_w = root @ hm
    mesh_w = root @ mesh_m
    expect = dict(sv=sv, rad=rad, pairs=pairs, mv=mv, mn=mn, tri=tri.reshape(-1, 3), hair_w=hair_w, mesh_w=mesh_w)
    return doc, bytes(blob), expect


def _check(prims, e, strip):
    hair = [p for p in prims if p.kind == "lines"]
    mesh = [p for p in prims if p.kind == "triangles"]
    assert len(hair) == (2 if strip else 1) and len(mesh) == 1
    for p, pairs in zip(hair, e["pairs"]):
        assert np.array_equal(p.vertices, e["sv"]) and np.array_equal(p.radius, e["rad"])
        assert np.array_equal(p.indices, pairs)
        assert np.allclose(p.transform, e["hair_w"], atol=1e-6)
    m = mesh[0]
    assert np.array_equal(m.vertices, e["mv"]) and np.array_equal(m.normals, e["mn"])
    assert np.array_equal(m.indices, e["tri"]) and np.allclose(m.transform, e["mesh_w"], atol=1e-7)
    assert m.blas_input().type == H.BLASType.eMesh
    assert hair[0].blas_input(H.BLASType.eLSS).type == H.BLASType.eLSS


@pytest.mark.parametrize("strip", [True, False])
@pytest.mark.parametrize("interleave", [True, False])
def test_gltf_external_buffer(tmp_path, strip, interleave):
    doc, blob, e = _doc_and_blob(strip, interleave)
    doc["buffers"][0]["uri"] = "model.bin"
    (tmp_path / "model.bin").write_bytes(blob)
    (tmp_path / "model.gltf").write_text(json.dumps(doc))
    _check(gltf.load(str(tmp_path / "model.gltf")), e, strip)


def test_gltf_data_uri_and_glb(tmp_path):
    doc, blob, e = _doc_and_blob(True, False)
    d1 = json.loads(json.dumps(doc))
    d1["buffers"][0]["uri"] = "data:application/octet-stream;base64," + base64.b64encode(blob).decode()
    (tmp_path / "a.gltf").write_text(json.dumps(d1))
    _check(gltf.load(str(tmp_path / "a.gltf")), e, True)
    js = json.dumps(doc).encode()
    js += b" " * (-len(js) % 4)
    bb = blob + b"\0" * (-len(blob) % 4)
    glb = struct.pack("<4sII", b"glTF", 2, 12 + 8 + len(js) + 8 + len(bb))
    glb += struct.pack("<II", len(js), 0x4E4F534A) + js + struct.pack("<II", len(bb), 0x004E4942) + bb
    (tmp_path / "a.glb").write_bytes(glb)
    _check(gltf.load(str(tmp_path / "a.glb")), e, True)


def test_gltf_errors(tmp_path):
    (tmp_path / "bad.gltf").write_text(json.dumps({"asset": {"version": "2.0"}, "nodes": [{"mesh": 0}],
                                                   "meshes": [{"primitives": [{"attributes": {}}]}]}))
    with pytest.raises(gltf.GltfError):
        gltf.load(str(tmp_path / "bad.gltf"))


def _png(img: np.ndarray) -> bytes:
    """An 8-bit PNG of img (h, w, c) whose rows use the filters None, Sub, Up, Average and Paeth in
    turn (the PNG specification's predictors), so that decoding undoes each of them."""
    import zlib
    h, w, c = img.shape
    ctype = {1: 0, 2: 4, 3: 2, 4: 6}[c]
    rows = img.reshape(h, w * c).astype(np.int32)
    out = bytearray()
    prev = np.zeros(w * c, np.int32)
    for y in range(h):
        f = y % 5
        cur = rows[y]
        a = np.concatenate([np.zeros(c, np.int32), cur[:-c]])
        b = prev
        cc = np.concatenate([np.zeros(c, np.int32), prev[:-c]])
        if f == 0:
            pred = np.zeros_like(cur)
        elif f == 1:
            pred = a
        elif f == 2:
            pred = b
        elif f == 3:
            pred = (a + b) >> 1
        else:
            pa, pb, pc = np.abs(b - cc), np.abs(a - cc), np.abs(a + b - 2 * cc)
            pred = np.where((pa <= pb) & (pa <= pc), a, np.where(pb <= pc, b, cc))
        out.append(f)
        out += ((cur - pred) & 255).astype(np.uint8).tobytes()
        prev = cur

    def chunk(kind, body):
        return struct.pack(">I", len(body)) + kind + body + struct.pack(">I", zlib.crc32(kind + body) & 0xFFFFFFFF)
    return (b"\x89PNG\r\n\x1a\n" + chunk(b"IHDR", struct.pack(">IIBBBBB", w, h, 8, ctype, 0, 0, 0)) +
            chunk(b"IDAT", zlib.compress(bytes(out))) + chunk(b"IEND", b""))


@pytest.mark.parametrize("channels", [1, 2, 3, 4])
def test_png_decoder_undoes_every_row_filter(channels):
    rng = np.random.default_rng(channels)
    img = rng.integers(0, 256, (11, 7, channels), dtype=np.uint8)
    got = gltf.decode_png(_png(img))
    assert got.shape == (11, 7, 4)
    want = np.ones((11, 7, 4), np.float32)
    px = img.astype(np.float32) / np.float32(255.0)
    if channels <= 2:
        want[..., :3] = px[..., :1]
        if channels == 2:
            want[..., 3] = px[..., 1]
    else:
        want[..., :channels] = px
    assert np.array_equal(got, want)


def test_gltf_mesh_material_and_texture(tmp_path):
    """A textured quad: TEXCOORD_0 (normalised unsigned shorts), the base colour factor and an
    embedded PNG base colour texture become the mesh BLAS's texcoords, albedo factor and map; an
    image that is not a PNG leaves the map out with a note."""
    v = np.array([[0, 0, 0], [1, 0, 0], [1, 1, 0], [0, 1, 0]], np.float32)
    idx = np.array([0, 1, 2, 0, 2, 3], np.uint16)
    tc = np.array([[0, 0], [65535, 0], [65535, 65535], [0, 65535]], np.uint16)
    blob = v.tobytes() + idx.tobytes() + tc.tobytes()
    img = np.random.default_rng(4).integers(0, 256, (3, 5, 4), dtype=np.uint8)
    png = _png(img)
    doc = {
        "asset": {"version": "2.0"}, "scene": 0, "scenes": [{"nodes": [0]}], "nodes": [{"mesh": 0}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0, "TEXCOORD_0": 2}, "indices": 1, "material": 0}]}],
        "materials": [{"pbrMetallicRoughness": {"baseColorFactor": [0.5, 0.25, 1.0, 1.0],
                                                "baseColorTexture": {"index": 0}}}],
        "textures": [{"source": 0}],
        "images": [{"uri": "data:image/png;base64," + base64.b64encode(png).decode()}],
        "buffers": [{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                     base64.b64encode(blob).decode()}],
        "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 48},
                        {"buffer": 0, "byteOffset": 48, "byteLength": 12},
                        {"buffer": 0, "byteOffset": 60, "byteLength": 16}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": 4, "type": "VEC3"},
                      {"bufferView": 1, "componentType": 5123, "count": 6, "type": "SCALAR"},
                      {"bufferView": 2, "componentType": 5123, "count": 4, "type": "VEC2", "normalized": True}],
    }
    path = tmp_path / "quad.gltf"
    path.write_text(json.dumps(doc))
    (p,) = gltf.load(str(path))
    assert p.kind == "triangles" and p.albedo_factor == (0.5, 0.25, 1.0, 1.0) and p.note == ""
    assert np.array_equal(p.texcoords, np.array([[0, 0], [1, 0], [1, 1], [0, 1]], np.float32))
    assert np.array_equal(p.albedo_map, img.astype(np.float32) / np.float32(255.0))
    inp = p.blas_input()
    assert inp.albedo_map is p.albedo_map and inp.texcoords is p.texcoords and inp.albedo_factor == p.albedo_factor
    doc["images"] = [{"uri": "data:image/jpeg;base64," + base64.b64encode(b"\xff\xd8\xff").decode()}]
    path.write_text(json.dumps(doc))
    (q,) = gltf.load(str(path))
    assert q.albedo_map is None and q.texcoords is None and "not a PNG" in q.note and q.albedo_factor[0] == 0.5


def test_gltf_material_factor_without_texture(tmp_path):
    """A material with a base colour factor and no texture: the factor alone, no texture
    coordinates or map."""
    v = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    blob = v.tobytes()
    doc = {
        "asset": {"version": "2.0"}, "nodes": [{"mesh": 0}],
        "meshes": [{"primitives": [{"attributes": {"POSITION": 0}, "material": 0}]}],
        "materials": [{"pbrMetallicRoughness": {"baseColorFactor": [0.2, 0.4, 0.6, 1.0]}}],
        "buffers": [{"byteLength": len(blob), "uri": "data:application/octet-stream;base64," +
                     base64.b64encode(blob).decode()}],
        "bufferViews": [{"buffer": 0, "byteOffset": 0, "byteLength": 36}],
        "accessors": [{"bufferView": 0, "componentType": 5126, "count": 3, "type": "VEC3"}],
    }
    path = tmp_path / "tri.gltf"
    path.write_text(json.dumps(doc))
    (p,) = gltf.load(str(path))
    assert p.albedo_factor == (0.2, 0.4, 0.6, 1.0) and p.albedo_map is None and p.texcoords is None
    assert p.indices.tolist() == [[0, 1, 2]]
