"""Generate the committed golden fixtures from the reference repository's assets.

Run where a checkout of the reference repository is available, giving its root:

    python tests/golden/make_golden.py <path to the lambdaxymox/bvhtracer checkout>

It parses the reference's ``bvhtracer/assets/cube.obj`` the way the reference's
ObjMeshDecoder does (BT/src/mesh/decoders.rs:157-215: one triangle per face,
corners in face order, per-corner normals from the ``//n`` index) and writes
``cube.npz`` (tris [12,9] f32, normals [12,9] f32).  It also decodes the
reference's mesh assets (``.tri`` / ``.obj``) with the library and with the Python
restatement of the reference's loaders and records counts, agreement and digests in
``assets.json``.  The GPU machine does not have the reference checkout, so tests read only
the committed fixtures.
"""
import os
import sys

import numpy as np


def parse_obj(text):
    vs, vns, faces = [], [], []
    for line in text.splitlines():
        parts = line.split()
        if not parts:
            continue
        if parts[0] == "v":
            vs.append([float(x) for x in parts[1:4]])
        elif parts[0] == "vn":
            vns.append([float(x) for x in parts[1:4]])
        elif parts[0] == "f":
            corner = []
            for c in parts[1:4]:
                fields = c.split("/")
                vi = int(fields[0]) - 1
                ni = int(fields[2]) - 1 if len(fields) > 2 and fields[2] else -1
                corner.append((vi, ni))
            faces.append(corner)
    tris = np.zeros((len(faces), 9), np.float32)
    normals = np.zeros((len(faces), 9), np.float32)
    for i, f in enumerate(faces):
        for k, (vi, ni) in enumerate(f):
            tris[i, 3 * k:3 * k + 3] = np.float32(vs[vi])
            if ni >= 0:
                normals[i, 3 * k:3 * k + 3] = np.float32(vns[ni])
    return tris, normals


ASSETS = ["bvhtracer/assets/cube.obj", "bvhtracer/tri_loader/assets/unity.tri", "examples/assets/triangle.tri",
          "examples/assets/unity.tri", "examples/assets/bigben.tri", "examples/assets/armadillo.tri",
          "examples/assets/cube.obj", "examples/assets/teapot.obj", "examples/assets/bunny.obj",
          "examples/assets/dragon.obj"]


def asset_digests(ref_root):
    """Decodes the reference's mesh assets with the library (bvhgpu_mesh_decode) and with the Python
    restatement (oracle/loaders.py), checks they agree bit for bit, and records counts and SHA-256
    digests of the decoded arrays (the assets themselves are not copied)."""
    import hashlib
    import json
    sys.path.insert(0, os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__)))))
    import bvhtracer_gb300 as bt
    from oracle import loaders as ol
    out = {}
    for rel in ASSETS:
        path = os.path.join(ref_root, rel)
        if not os.path.exists(path):
            continue
        with open(path, "rb") as f:
            raw = f.read()
        obj = rel.endswith(".obj")
        text = raw.decode("utf-8", errors="replace")
        try:
            mine = bt.decode_mesh(raw, bt.MESH_OBJ if obj else bt.MESH_TRI)
        except bt.BvhGpuError as e:
            mine = e
        try:
            ref = ol.decode_obj(text) if obj else ol.decode_tri(text)
        except (ValueError, IndexError) as e:
            ref = e
        if isinstance(mine, Exception) or isinstance(ref, Exception):
            out[rel] = {"error_library": str(mine) if isinstance(mine, Exception) else None,
                        "error_restatement": str(ref) if isinstance(ref, Exception) else None}
            continue
        same = all(a.tobytes() == b.tobytes() for a, b in zip(mine, ref))
        out[rel] = {"triangles": int(len(mine[0])), "identical_to_restatement": bool(same),
                    "sha256_tris": hashlib.sha256(mine[0].tobytes()).hexdigest(),
                    "sha256_normals": hashlib.sha256(mine[1].tobytes()).hexdigest(),
                    "sha256_uvs": hashlib.sha256(mine[2].tobytes()).hexdigest()}
        print(rel, out[rel].get("triangles"), "identical" if same else "DIFFERENT")
    return out


def main(ref_root):
    import json
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(ref_root, "bvhtracer", "assets", "cube.obj")) as f:
        tris, normals = parse_obj(f.read())
    np.savez(os.path.join(here, "cube.npz"), tris=tris, normals=normals)
    print("cube:", tris.shape)
    with open(os.path.join(here, "assets.json"), "w") as f:
        json.dump(asset_digests(ref_root), f, indent=1, sort_keys=True)


if __name__ == "__main__":
    if len(sys.argv) != 2:
        sys.exit("usage: make_golden.py <path to the reference checkout>")
    main(sys.argv[1])
