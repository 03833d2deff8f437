"""Readers and writers of BVHTest's on-disk formats (used to feed the `load`, `camImport` and
`BVHImport` commands and to read what `BVHExport` / `writeData` produce).

* mesh v3 (lib/io/Load.cpp:122-139): data.json {"version": 3, "bin": ..., "mesh": {"vert", "normals",
  "faces"}} + raw float3 vert[], float3 norm[], uint3 faces[];
* cameras v1 (lib/io/CameraImport.cpp:42-108): cameras.json {"version": 1, "cameras": [{"type":
  "PERSPECTIVE", "cam": {"camera": {pos, lookAt, up, fov}, "resolution": {width, height}}}]};
* BVH v9 (lib/io/BVHExport.cpp:44-117): <name>_bvh.json {"version": 9, "bin", "BVHSize", "treeHeight",
  "rawChecksum" (adler32)} + raw 48-byte nodes.
"""
from __future__ import annotations

import json
import zlib
from pathlib import Path

import numpy as np

from .native import NODE_DTYPE


def write_mesh_v3(directory, vert, faces, norm=None, bin_name="data.bin"):
    d = Path(directory)
    d.mkdir(parents=True, exist_ok=True)
    vert = np.ascontiguousarray(vert, np.float32).reshape(-1, 3)
    faces = np.ascontiguousarray(faces, np.uint32).reshape(-1, 3)
    norm = np.zeros((0, 3), np.float32) if norm is None else np.ascontiguousarray(norm, np.float32).reshape(-1, 3)
    (d / bin_name).write_bytes(vert.tobytes() + norm.tobytes() + faces.tobytes())
    meta = {"version": 3, "bin": bin_name,
            "mesh": {"vert": int(vert.shape[0]), "normals": int(norm.shape[0]), "faces": int(faces.shape[0])}}
    (d / "data.json").write_text(json.dumps(meta, indent=2))
    return d / "data.json"


def write_cameras_v1(directory, cameras):
    cams = []
    for c in cameras:
        v = lambda p: {"x": float(p[0]), "y": float(p[1]), "z": float(p[2])}  # noqa: E731
        cams.append({"type": "PERSPECTIVE",
                     "cam": {"camera": {"pos": v(c["pos"]), "lookAt": v(c["lookAt"]), "up": v(c["up"]),
                                        "fov": float(c["fov"])},
                             "resolution": {"width": int(c["width"]), "height": int(c["height"])}}})
    p = Path(directory) / "cameras.json"
    p.write_text(json.dumps({"version": 1, "cameras": cams}, indent=2))
    return p


def read_bvh_v9(directory, name="genericBVH"):
    d = Path(directory)
    meta = json.loads((d / f"{name}_bvh.json").read_text())
    if meta["version"] != 9:
        raise ValueError("BVH format version %s, 9 required" % meta["version"])
    raw = (d / meta["bin"]).read_bytes()
    if zlib.adler32(raw) != meta["rawChecksum"]:
        raise ValueError("corrupt BVH binary")
    nodes = np.frombuffer(raw, NODE_DTYPE).copy()
    assert nodes.shape[0] == meta["BVHSize"]
    return nodes, meta


def write_bvh_v9(directory, nodes, name="genericBVH", tree_height=0):
    d = Path(directory)
    raw = np.ascontiguousarray(nodes).view(np.uint8).tobytes()
    (d / f"{name}_bvh.bin").write_bytes(raw)
    meta = {"version": 9, "bin": f"{name}_bvh.bin", "BVHSize": int(len(raw) // 48), "treeHeight": int(tree_height),
            "rawChecksum": zlib.adler32(raw)}
    (d / f"{name}_bvh.json").write_text(json.dumps(meta, indent=2))
