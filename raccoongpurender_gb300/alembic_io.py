"""Write scenes as Alembic (Ogawa) archives in the shape a Houdini export has:
every object under its own transform, triangle meshes with per-primitive
"material" and property columns as geometry parameters, point objects with
per-point columns, a camera with Houdini's resx / resy user properties.
Files written here load with ``SceneManager.addAlembic`` and with the
reference's own reader (libs/houdini_alembic on the Alembic SDK).

The container: a 16-byte header ("Ogawa", frozen flag 0xff, version 1, root
group offset), then data blocks (64-bit size + bytes) and groups (64-bit
child count + child offsets; a data child has the top bit set), children
before parents.  The Alembic layout on it: the archive root group holds the
file version, the library version, the top object, the archive metadata, the
time samplings and the indexed metadata; an object group holds its property
compound, its child objects and a block of child headers followed by two
16-byte digests; a compound holds one group per property and a block of
packed property headers; a sample is a data block led by a 16-byte digest,
an array sample adds a block of 64-bit dimensions.  Every property written
here has one sample (a static scene: frame 0).
"""
from __future__ import annotations

import hashlib
import struct
from pathlib import Path

import numpy as np

_DATA = 1 << 63
# POD codes (AbcCoreAbstract PlainOldDataType)
_U8, _I8, _U32, _I32, _U64, _F32, _F64, _STR = 1, 2, 5, 6, 7, 10, 11, 12
_OPS = {"scale": 0, "translate": 1, "rotate": 2, "matrix": 3, "rotate_x": 4, "rotate_y": 5, "rotate_z": 6}


def _meta(d: dict) -> str:
    return ";".join(f"{k}={d[k]}" for k in sorted(d))


class _Ogawa:
    def __init__(self):
        self.buf = bytearray(b"Ogawa" + bytes([0xFF, 0, 1]) + bytes(8))

    def data(self, payload: bytes) -> int:
        if len(payload) == 0:
            return _DATA
        pos = len(self.buf)
        self.buf += struct.pack("<Q", len(payload)) + payload
        return pos | _DATA

    def group(self, children) -> int:
        if not children:
            return 0
        pos = len(self.buf)
        self.buf += struct.pack("<Q", len(children)) + struct.pack(f"<{len(children)}Q", *children)
        return pos

    def finish(self, root: int) -> bytes:
        self.buf[8:16] = struct.pack("<Q", root)
        return bytes(self.buf)


def _hint(values) -> int:
    m = max(values)
    return 0 if m < 256 else (1 if m < 65536 else 2)


def _pack_hint(v: int, hint: int) -> bytes:
    return struct.pack("<B" if hint == 0 else ("<H" if hint == 1 else "<I"), v)


class _Compound:
    """Properties of one compound, written as they are added."""

    def __init__(self, o: _Ogawa):
        self.o = o
        self.entries = []
        self.headers = bytearray()

    def _header(self, name: str, ptype: int, meta: dict, pod: int = 0, extent: int = 1) -> None:
        m = _meta(meta)
        hint = _hint([len(m), len(name), 1])
        info = (hint << 2) | ((0xFF if m else 0) << 20)
        tail = b""
        if ptype != 0:
            # one sample, all samples equal (first = last changed = 0)
            info |= ptype | (pod << 4) | 0x800 | (extent << 12) | 0x400
            tail += _pack_hint(1, hint)
        tail += _pack_hint(len(name), hint) + name.encode()
        if m:
            tail += _pack_hint(len(m), hint) + m.encode()
        self.headers += struct.pack("<I", info) + tail

    def _sample(self, payload: bytes) -> int:
        return self.o.data(hashlib.md5(payload).digest() + payload if payload else b"")

    def scalar(self, name: str, pod: int, values: bytes, extent: int, meta: dict | None = None) -> None:
        self._header(name, 1, meta or {}, pod, extent)
        self.entries.append(self.o.group([self._sample(values)]))

    def array(self, name: str, arr, meta: dict | None = None) -> None:
        """A float32 / int32 / uint32 / uint64 array (extent = its second axis) or a list of strings."""
        if isinstance(arr, (list, tuple)) and (len(arr) == 0 or isinstance(arr[0], str)):
            pod, extent, count = _STR, 1, len(arr)
            payload = b"".join(s.encode() + b"\0" for s in arr)
        else:
            a = np.ascontiguousarray(arr)
            pod = {np.dtype(np.float32): _F32, np.dtype(np.int32): _I32, np.dtype(np.uint32): _U32,
                   np.dtype(np.uint64): _U64, np.dtype(np.float64): _F64}[a.dtype]
            extent = 1 if a.ndim == 1 else int(a.shape[1])
            count = int(a.shape[0])
            payload = a.astype(a.dtype.newbyteorder("<")).tobytes()
        self._header(name, 2, meta or {}, pod, extent)
        dims = self.o.data(struct.pack("<Q", count))
        self.entries.append(self.o.group([self._sample(payload), dims]))

    def compound(self, name: str, meta: dict | None = None) -> "_Compound":
        c = _Compound(self.o)
        self._header(name, 0, meta or {})
        self.entries.append(c)  # written when this compound is closed
        return c

    def close(self) -> int:
        kids = [e.close() if isinstance(e, _Compound) else e for e in self.entries]
        return self.o.group(kids + [self.o.data(bytes(self.headers))])


class _Object:
    def __init__(self, o: _Ogawa, name: str, meta: dict):
        self.o, self.name, self.meta = o, name, meta
        self.props = _Compound(o)
        self.children = []

    def child(self, name: str, meta: dict) -> "_Object":
        c = _Object(self.o, name, meta)
        self.children.append(c)
        return c

    def close(self) -> int:
        props = self.props.close()
        kids = [c.close() for c in self.children]
        hdr = bytearray()
        for c in self.children:
            m = _meta(c.meta).encode()
            hdr += struct.pack("<I", len(c.name)) + c.name.encode() + bytes([0xFF]) + struct.pack("<I", len(m)) + m
        hdr += bytes(32)  # the data and children digests
        return self.o.group([props] + kids + [self.o.data(bytes(hdr))])


def _geom_param(c: _Compound, name: str, values, scope: str) -> None:
    """A geometry parameter: strings indexed (a compound of .vals and .indices),
    float32 / int32 arrays as they are (extent = the second axis)."""
    if isinstance(values, (list, tuple)) and values and isinstance(values[0], str):
        uniq = sorted(set(values))
        lut = {s: i for i, s in enumerate(uniq)}
        meta = dict(arrayExtent=1, geoScope=scope, interpretation="", isGeomParam="true", podExtent=1,
                    podName="string")
        g = c.compound(name, meta)
        g.array(".vals", uniq, meta)
        g.array(".indices", np.asarray([lut[s] for s in values], np.uint32))
        return
    a = np.ascontiguousarray(values)
    ext = 1 if a.ndim == 1 else a.shape[1]
    pod = "float32_t" if a.dtype == np.float32 else "int32_t"
    c.array(name, a, dict(arrayExtent=1, geoScope=scope, interpretation="", isGeomParam="true", podExtent=ext,
                          podName=pod))


def _xform(top: _Object, name: str, ops) -> _Object:
    xf = top.child(name, dict(schema="AbcGeom_Xform_v3", schemaObjTitle="AbcGeom_Xform_v3:.xform"))
    xf.props.scalar("visible", _I8, struct.pack("<b", -1), 1)
    x = xf.props.compound(".xform", dict(schema="AbcGeom_Xform_v3"))
    x.scalar(".inherits", 0, b"\x01", 1)
    codes, vals = [], []
    for op, v in ops or []:
        codes.append(_OPS[op] << 4)
        vals.extend(float(t) for t in np.asarray(v, np.float64).ravel())
    if codes:
        x.scalar(".ops", _U8, bytes(codes), len(codes))
        x.scalar(".vals", _F64, struct.pack(f"<{len(vals)}d", *vals), len(vals))
    return xf


def _bounds(P) -> bytes:
    P = np.asarray(P, np.float64).reshape(-1, 3)
    lo, hi = (P.min(0), P.max(0)) if len(P) else (np.zeros(3), np.zeros(3))
    return struct.pack("<6d", *lo, *hi)


_MAT_NAMES = {1: "Lambertian", 2: "Specular", 3: "Dierectric", 4: "Ward", 5: "HomogeneousVolume"}


def columns_from_materials(mats) -> dict:
    """Per-primitive columns (material names and their properties, as
    SceneManager's add_materials reads them) from a MATERIAL_DTYPE array."""
    m = np.asarray(mats)
    t = m["type"]
    lam, ward, vol = t == 1, t == 4, t == 5
    cd = np.where((lam | vol)[:, None], m["r"], np.float32(1.0)).astype(np.float32)
    return {"material": [_MAT_NAMES[int(k)] for k in t],
            "Le": np.ascontiguousarray(m["le"], np.float32),
            "Cd": cd,
            "BackEmission": np.ascontiguousarray(m["back_emission"], np.int32),
            "reflectance": np.where(ward[:, None], m["r"], np.float32(1.0)).astype(np.float32),
            "edgetint": np.ascontiguousarray(m["edgetint"], np.float32),
            "alpha": np.ascontiguousarray(m["alpha"], np.float32),
            "falloff": np.ascontiguousarray(m["falloff"], np.float32),
            "C": np.ascontiguousarray(m["c"], np.float32)}


def write_scene(path, meshes=(), points=(), camera=None) -> int:
    """Write an archive; returns its size in bytes.

    meshes: dicts with name, P (n, 3) float32, indices (t, 3) uint32, and
        optionally ops (transform ops: ("translate", xyz), ("scale", xyz),
        ("rotate", (ax, ay, az, degrees)), ("rotate_x"|"rotate_y"|"rotate_z", deg),
        ("matrix", 4x4 in Imath's row-vector layout)) and prims: {column:
        per-triangle values}, e.g. material (names), Cd / Le (t, 3) float32,
        alpha (t,) float32, BackEmission (t,) int32.
    points: dicts with name, P, ops, and cols: {column: per-point values}
        (pscale, Cd, or point_type / file / clamp / scale for an envmap).
    camera: dict with ops, focal_mm, aperture_h_cm, aperture_v_cm,
        focus_distance, f_stop, resx, resy.
    """
    o = _Ogawa()
    top = _Object(o, "", {})
    geo = dict(schema="AbcGeom_PolyMesh_v1", schemaBaseType="AbcGeom_GeomBase_v1",
               schemaObjTitle="AbcGeom_PolyMesh_v1:.geom")
    for m in meshes:
        xf = _xform(top, m["name"], m.get("ops"))
        ob = xf.child(m["name"] + "Shape", geo)
        g = ob.props.compound(".geom", dict(schema="AbcGeom_PolyMesh_v1", schemaBaseType="AbcGeom_GeomBase_v1"))
        P = np.ascontiguousarray(m["P"], np.float32).reshape(-1, 3)
        idx = np.ascontiguousarray(m["indices"], np.uint32).reshape(-1, 3)
        g.scalar(".selfBnds", _F64, _bounds(P), 6, dict(interpretation="box"))
        g.array("P", P, dict(geoScope="vtx", interpretation="point"))
        g.array(".faceIndices", idx.reshape(-1).astype(np.int32))
        g.array(".faceCounts", np.full(idx.shape[0], 3, np.int32))
        arb = g.compound(".arbGeomParams")
        for k, v in (m.get("prims") or {}).items():
            _geom_param(arb, k, v, "uni")
    pts = dict(schema="AbcGeom_Points_v1", schemaBaseType="AbcGeom_GeomBase_v1",
               schemaObjTitle="AbcGeom_Points_v1:.geom")
    for p in points:
        xf = _xform(top, p["name"], p.get("ops"))
        ob = xf.child(p["name"] + "Shape", pts)
        g = ob.props.compound(".geom", dict(schema="AbcGeom_Points_v1", schemaBaseType="AbcGeom_GeomBase_v1"))
        P = np.ascontiguousarray(p["P"], np.float32).reshape(-1, 3)
        g.scalar(".selfBnds", _F64, _bounds(P), 6, dict(interpretation="box"))
        g.array("P", P, dict(geoScope="var", interpretation="point"))
        g.array(".pointIds", np.arange(P.shape[0], dtype=np.uint64))
        arb = g.compound(".arbGeomParams")
        for k, v in (p.get("cols") or {}).items():
            _geom_param(arb, k, v, "var")
    if camera is not None:
        xf = _xform(top, "cam", camera.get("ops"))
        ob = xf.child("camShape", dict(schema="AbcGeom_Camera_v1", schemaObjTitle="AbcGeom_Camera_v1:.geom"))
        g = ob.props.compound(".geom", dict(schema="AbcGeom_Camera_v1"))
        core = [camera.get("focal_mm", 35.0), camera.get("aperture_h_cm", 3.6), 0.0, camera.get("aperture_v_cm", 2.4),
                0.0, 1.0, 0.0, 0.0, 0.0, 0.0, camera.get("f_stop", 5.6), camera.get("focus_distance", 5.0),
                0.0, 0.0, 0.1, 100000.0]
        g.scalar(".core", _F64, struct.pack("<16d", *core), 16)
        up = g.compound(".userProperties")
        up.scalar("resx", _F32, struct.pack("<f", float(camera["resx"])), 1)
        up.scalar("resy", _F32, struct.pack("<f", float(camera["resy"])), 1)
    top_entry = top.close()
    root = o.group([
        o.data(struct.pack("<i", 0)),                  # file version
        o.data(struct.pack("<i", 10709)),              # library version
        top_entry,
        o.data(b"_ai_Application=raccoongpurender_gb300"),
        o.data(struct.pack("<IdId", 0, 1.0, 1, 0.0)),  # time sampling 0: identity
        o.data(b""),                                    # no indexed metadata
    ])
    out = o.finish(root)
    Path(path).write_bytes(out)
    return len(out)
