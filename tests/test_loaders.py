"""Mesh decoders (bvhgpu_mesh_decode) against the Python restatement in oracle/loaders.py and the
reference loader's own test vectors (bvhtracer/tri_loader/src/loader.rs tests); the `.obj` path
against the committed cube fixture.  CPU only."""
import numpy as np
import pytest

import bvhtracer_gb300 as bt
from oracle import loaders as ol

# tri_loader/src/loader.rs: test_lexer_one_line / test_lexer_multiple_lines (lines end in '\\')
ONE_LINE = "\n            -1.920570 0.000680 0.030130 -1.927750 0.102380 0.000170 -1.965040 0.013640 0.009820\n        "
MULTI = """
            -1.920570 0.000680 0.030130 -1.927750 0.102380 0.000170 -1.965040 0.013640 0.009820     \\
            -1.879360 0.093640 0.019450 -1.927750 0.102380 0.000170 -1.920570 0.000680 0.030130     \\
            -1.879360 0.093640 0.019450 -1.889650 0.172390 -0.028960 -1.927750 0.102380 0.000170    \\
            -1.838710 0.162240 -0.008080 -1.889650 0.172390 -0.028960 -1.879360 0.093640 0.019450   \\
            -1.838710 0.162240 -0.008080 -1.844990 0.231520 -0.074300 -1.889650 0.172390 -0.028960  \\
                                                                                                    \\
                                                                                                    \\
        """


def same(a, b):
    return all(x.tobytes() == y.tobytes() for x, y in zip(a, b))


def test_reference_loader_vectors():
    assert bt.decode_mesh("")[0].shape == (0, 9)
    t, n, uv = bt.decode_mesh(ONE_LINE)
    assert t.shape == (1, 9)
    assert t[0].tolist() == np.array([-1.920570, 0.000680, 0.030130, -1.927750, 0.102380, 0.000170,
                                      -1.965040, 0.013640, 0.009820], np.float32).tolist()
    t5, n5, _ = bt.decode_mesh(MULTI)
    assert t5.shape == (5, 9)
    assert t5[3].tolist() == np.array([-1.838710, 0.162240, -0.008080, -1.889650, 0.172390, -0.028960,
                                       -1.879360, 0.093640, 0.019450], np.float32).tolist()
    assert same(bt.decode_mesh(MULTI), ol.decode_tri(MULTI))
    assert np.all(uv == 0)
    assert np.allclose(np.linalg.norm(n5.reshape(-1, 3), axis=1), 1, atol=1e-6)


def test_tokens_comments_and_float_grammar():
    text = ("# header comment\n\n\t1 2 3 4 5 6 7 8 9   # trailing\n"
            "+1. .5 -0.0 1e-45 3.4028236e38 1E+2 inf -Infinity NaN\n"
            "\\ 0.1 0.2 0.3\t0.4 0.5 0.6 0.7 0.8 0.9\\\n\n\n")
    got, ref = bt.decode_mesh(text), ol.decode_tri(text)
    assert got[0].shape == (3, 9)
    assert got[0].tobytes() == ref[0].tobytes()                    # every bit, NaN and -0 included
    assert got[0][1, 3] == np.float32(1e-45) and got[0][1, 4] == np.inf   # subnormal, overflow
    assert np.signbit(got[0][1, 2]) and got[0][1, 7] == -np.inf
    assert got[1][0].tobytes() == ref[1][0].tobytes() and got[1][2].tobytes() == ref[1][2].tobytes()


@pytest.mark.parametrize("text,line,kind", [
    ("1 2 3 4 5 6 7 8 x\n", 1, "ExpectedFloat"),
    ("1 2 3 4 5 6 7 8 9\n1 2 3\n4 5 6 7 8 9\n", 3, "ExpectedFloat"),   # a newline inside a triangle
    ("1 2 3 4 5 6 7 8 9\r\n", 1, "ExpectedFloat"),                   # '\r' is a token of its own
    ("1 2 3 4 5 6 7 8", 1, "EndOfFile"),
    ("1 2 3 4 5 6 7 8 0x10\n", 1, "ExpectedFloat"),                 # no hex floats in Rust
    ("1 2 3 4 5 6 7 8 1e\n", 1, "ExpectedFloat"),
])
def test_errors_match_the_reference_loader(text, line, kind):
    with pytest.raises(ol.DecodeError) as e:
        ol.decode_tri(text)
    assert (e.value.line, e.value.kind) == (line, kind)
    with pytest.raises(bt.BvhGpuError) as g:
        bt.decode_mesh(text)
    assert f"line {line}: {kind}" in str(g.value)


def test_random_tri_files_match_the_oracle():
    rng = np.random.default_rng(7)
    v = (rng.standard_normal((300, 9)) * 10 ** rng.uniform(-6, 6, (300, 1))).astype(np.float32)
    fmts = ["{:.9g}", "{:.3f}", "{:e}", "{:.12g}"]
    lines = []
    for k, row in enumerate(v):
        f = fmts[k % len(fmts)]
        lines.append((" " if k % 2 else "\t").join(f.format(float(x)) for x in row))
    text = "\n\n".join(lines) + "\n"
    got, ref = bt.decode_mesh(text), ol.decode_tri(text)
    assert same(got, ref)
    exact = bt.decode_mesh("\n".join(" ".join("{:.9g}".format(float(x)) for x in r) for r in v))[0]
    assert exact.tobytes() == v.tobytes()                            # 9 significant digits round-trip


def cube_obj():
    import os
    d = np.load(os.path.join(os.path.dirname(__file__), "golden", "cube.npz"))
    tris, normals = d["tris"], d["normals"]
    out = ["# cube, one vertex and one normal per corner", "g cube"]
    for t, n in zip(tris, normals):
        for k in range(3):
            out.append("v {:.9g} {:.9g} {:.9g}".format(*map(float, t[3 * k:3 * k + 3])))
            out.append("vn {:.9g} {:.9g} {:.9g}".format(*map(float, n[3 * k:3 * k + 3])))
    for i in range(len(tris)):
        out.append("f " + " ".join(f"{3 * i + k + 1}//{3 * i + k + 1}" for k in range(3)))
    return "\n".join(out) + "\n", tris, normals


def test_obj_cube_and_features():
    text, tris, normals = cube_obj()
    t, n, uv = bt.decode_mesh(text, bt.MESH_OBJ)
    assert t.tobytes() == tris.tobytes() and n.tobytes() == normals.tobytes() and np.all(uv == 0)
    assert same((t, n, uv), ol.decode_obj(text))
    quad = ("v 0 0 0\nv 1 0 0\nv 1 1 0\nv 0 1 0\nvt 0 0\nvt 1 0\nvt 1 1\nvt 0 1\nvn 0 0 1\n"
            "f 1/1/1 2/2/1 3/3/1 4/4/1\nf -4/-4 -2/-2 -1/-1\no second\nv 5 5 5\nf 1 2 3\n")
    got = bt.decode_mesh(quad, bt.MESH_OBJ)
    assert got[0].shape == (3, 9)                                   # fan of the quad + 1; object 2 dropped
    assert same(got, ol.decode_obj(quad))
    with pytest.raises(bt.BvhGpuError):
        bt.decode_mesh("v 0 0 0\nf 1 2 3\n", bt.MESH_OBJ)           # index out of range


def test_decode_file(tmp_path):
    p = tmp_path / "five.tri"
    p.write_text(MULTI)
    assert same(bt.load_mesh(str(p)), ol.decode_tri(MULTI))


def test_reference_assets_were_decoded_identically():
    """tests/golden/assets.json, written by make_golden.py from the reference's ten mesh assets
    (unity, bigben, armadillo, teapot, bunny, dragon, cube, ...): the library's decode equals the
    Python restatement's bit for bit, and the library's decode of the reference's cube.obj is the
    cube fixture the known-answer tests use."""
    import hashlib
    import json
    import os
    here = os.path.join(os.path.dirname(__file__), "golden")
    with open(os.path.join(here, "assets.json")) as f:
        d = json.load(f)
    assert len(d) >= 10
    assert all(v.get("identical_to_restatement") for v in d.values())
    assert d["examples/assets/armadillo.tri"]["triangles"] == 30001
    cube = np.load(os.path.join(here, "cube.npz"))
    assert d["bvhtracer/assets/cube.obj"]["sha256_tris"] == hashlib.sha256(cube["tris"].tobytes()).hexdigest()
    assert d["bvhtracer/assets/cube.obj"]["sha256_normals"] == hashlib.sha256(cube["normals"].tobytes()).hexdigest()
