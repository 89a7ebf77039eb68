"""Generate the committed golden fixtures from the reference repository's assets.

Run in a container that has the reference checkout (read-only) mounted:

    python tests/golden/make_golden.py /root/reference

It parses the reference's ``bvhtracer/assets/cube.obj`` the way the reference's
ObjMeshDecoder does (BT/src/mesh/decoders.rs:157-215: one triangle per face,
corners in face order, per-corner normals from the ``//n`` index) and writes
``cube.npz`` (tris [12,9] f32, normals [12,9] f32).  The GPU machine does not have
the reference checkout, so tests read only the committed ``.npz``.
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


def main(ref_root):
    here = os.path.dirname(os.path.abspath(__file__))
    with open(os.path.join(ref_root, "bvhtracer", "assets", "cube.obj")) as f:
        tris, normals = parse_obj(f.read())
    np.savez(os.path.join(here, "cube.npz"), tris=tris, normals=normals)
    print("cube:", tris.shape)


if __name__ == "__main__":
    main(sys.argv[1] if len(sys.argv) > 1 else "/root/reference")
