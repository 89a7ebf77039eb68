"""Whole-scene render through the C ABI (bvhgpu_render_scene: Integrator::evaluate for PathTracer on a
Scene, renderer.rs:345-384 -> Scene::intersect) against the oracle's restatement (orc_render_scene).

Scenes: the reference's cube scene (assets/cube.obj under Transform3::new(scale 2, translate -1),
camera at (0, 4, 0) looking down, tests/test_scene_cube.rs:28-83) and a multi-instance scene of three
displaced icospheres under random rotations, scales and translations.  Every accumulator x shader, and
for the normal / texture accumulators both lookups: the reference's (object 0's model and transform
for every hit, because its Bvh::intersect packs instance 0) and the hit's own object.  Bar: images
identical byte for byte.
"""
import os

import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes
from oracle import checks
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
HERE = os.path.dirname(__file__)


@pytest.fixture(scope="module")
def ctx():
    c = bt.Context(0)
    yield c
    c.close()


def random_instances(n, seed, spread=6.0):
    rng = np.random.default_rng(seed)
    q = rng.standard_normal((n, 4))
    q /= np.linalg.norm(q, axis=1, keepdims=True)
    w, x, y, z = q.T
    R = np.stack([np.stack([1 - 2 * (y * y + z * z), 2 * (x * y - w * z), 2 * (x * z + w * y)], -1),
                  np.stack([2 * (x * y + w * z), 1 - 2 * (x * x + z * z), 2 * (y * z - w * x)], -1),
                  np.stack([2 * (x * z - w * y), 2 * (y * z + w * x), 1 - 2 * (x * x + y * y)], -1)], 1)
    s = rng.uniform(0.5, 2.0, n)
    t = rng.uniform(-spread, spread, (n, 3))
    M = np.zeros((n, 4, 4))
    M[:, :3, :3] = R * s[:, None, None]
    M[:, :3, 3] = t
    M[:, 3, 3] = 1
    inv = np.linalg.inv(M)
    return (np.ascontiguousarray(M.transpose(0, 2, 1).reshape(n, 16), np.float32),
            np.ascontiguousarray(inv.transpose(0, 2, 1).reshape(n, 16), np.float32))


def shaded_mesh(level, seed):
    """A displaced icosphere built by the reference's SAH build, with its per-corner normals (the
    vertices' unit directions) and spherical texture coordinates in the build's triangle order."""
    mesh = scenes.displaced_icosphere(level, seed)
    tris0 = mesh.triangles()
    nrm0 = np.ascontiguousarray(mesh.dirs[mesh.faces].reshape(-1, 9).astype(np.float32))
    d = mesh.dirs
    uv = np.stack([np.arctan2(d[:, 2], d[:, 0]) / (2 * np.pi) * 3.0 + 0.5,
                   np.arccos(np.clip(d[:, 1], -1, 1)) / np.pi * 2.0 - 0.25], 1).astype(np.float32)
    tc0 = np.ascontiguousarray(uv[mesh.faces].reshape(-1, 6))
    tris, nodes, used = orc.bvh_build(tris0)
    order = {t.tobytes(): i for i, t in enumerate(tris0)}
    perm = np.array([order[t.tobytes()] for t in tris])
    return tris, nodes, used, nrm0[perm], tc0[perm]


CASES = [(bt.ACC_INTERSECTION, bt.SHADER_INTERSECTION), (bt.ACC_INTERSECTION, bt.SHADER_RADIANCE),
         (bt.ACC_DEPTH, bt.SHADER_DEPTH), (bt.ACC_UV, bt.SHADER_RADIANCE), (bt.ACC_NORMAL, bt.SHADER_RADIANCE),
         (bt.ACC_TEXTURE, bt.SHADER_RADIANCE), (bt.ACC_NORMAL, bt.SHADER_INTERSECTION)]
ACC_PARAMS = [0.2, 0.6, 1.0, 0.0, 0.0, 0.0]
SHADER_PARAMS = {bt.SHADER_INTERSECTION: [255, 255, 255, 255, 0, 0, 0, 255], bt.SHADER_DEPTH: [40.0, 1.0]}


def render_both(ctx, sc, blas_states, blas_of, shading, cam, w, h, acc, shader, lookup):
    xf, inv = sc.download_transforms()
    tlas, used = sc.download_tlas()
    ref_tlas, ref_used, sa = checks.scene_state_reference(blas_states, blas_of, xf, inv)
    assert used == ref_used and tlas.tobytes() == ref_tlas.tobytes()
    ap = ACC_PARAMS if acc == bt.ACC_INTERSECTION else None
    sp = SHADER_PARAMS.get(shader)
    rgba, n = sc.render(cam, w, h, acc, shader, ap, sp, lookup=lookup)
    ref, _ = orc.render_scene(cam.corners(), cam.view_inv, w, h, ref_tlas, sa, xf, acc, shader, acc_params=ap,
                              shader_params=sp, normals=[s[0] for s in shading],
                              tex_coords=[s[1] for s in shading], textures=[s[2] for s in shading], lookup=lookup)
    assert n == w * h
    return rgba, ref


@pytest.mark.parametrize("acc,shader", CASES)
def test_cube_scene_render_matches_oracle(ctx, acc, shader):
    d = np.load(os.path.join(HERE, "golden", "cube.npz"))
    tris0 = d["tris"]
    tris, nodes, used = orc.bvh_build(tris0)
    order = {t.tobytes(): i for i, t in enumerate(tris0)}
    perm = np.array([order[t.tobytes()] for t in tris])
    nrm = d["normals"][perm]
    tc = np.ascontiguousarray(np.tile(np.array([[0.1, 0.2, 0.9, 0.3, 0.4, 0.8]], np.float32), (len(tris), 1)) +
                              np.arange(len(tris), dtype=np.float32)[:, None] * 0.05)
    tex = np.random.default_rng(1).integers(0, 256, (16, 16, 3), dtype=np.uint8)
    blas = ctx.upload_blas(bt.Bvh(nodes, used), tris)
    blas.set_shading(nrm, tc, tex)
    # Transform3::new(scale 2, translate -1, identity rotation) (test_scene_cube.rs:53-65)
    xf = np.eye(4, dtype=np.float32)
    xf[:3, :3] *= 2
    xf[3, :3] = -1
    inv = np.eye(4, dtype=np.float32)
    inv[:3, :3] *= 0.5
    inv[3, :3] = 0.5
    sc = ctx.scene([blas], xf.reshape(1, 16), inv.reshape(1, 16))
    # camera at (0, 4, 0) looking at the origin, right -x, up +z (test_scene_cube.rs:29-47)
    cam = bt.Camera((-1, 1, -1, 1, 1, 100), (0, 4, 0), (0, -1, 0), (-1, 0, 0), (0, 0, 1))
    for lookup in (bt.LOOKUP_REFERENCE, bt.LOOKUP_HIT_OBJECT):
        rgba, ref = render_both(ctx, sc, [(nodes[:used], used, tris)], np.zeros(1, np.uint32), [(nrm, tc, tex)],
                                cam, 160, 120, acc, shader, lookup)
        assert np.array_equal(rgba, ref), f"lookup {lookup}: {np.count_nonzero(rgba != ref)} bytes differ"
    assert len(np.unique(rgba.reshape(-1, 4), axis=0)) >= 2
    sc.free()


@pytest.fixture(scope="module")
def instanced(ctx):
    """Three displaced icospheres (levels 3, 2, 1) and 24 instances; object 0 uses the largest."""
    meshes = [shaded_mesh(lvl, 20 + lvl) for lvl in (3, 2, 1)]
    blases, states, shading = [], [], []
    rng = np.random.default_rng(3)
    for k, (tris, nodes, used, nrm, tc) in enumerate(meshes):
        b = ctx.upload_blas(bt.Bvh(nodes, used), tris)
        tex = rng.integers(0, 256, (9 + 4 * k, 13 + 2 * k, 3), dtype=np.uint8)
        b.set_shading(nrm, tc, tex)
        blases.append(b)
        states.append((nodes[:used], used, tris))
        shading.append((nrm, tc, tex))
    n = 24
    blas_of = (np.arange(n) % 3).astype(np.uint32)
    xf, inv = random_instances(n, 11)
    sc = ctx.scene([blases[i] for i in blas_of], xf, inv)
    yield sc, states, blas_of, shading, blases
    sc.free()


@pytest.mark.parametrize("acc,shader", CASES)
def test_instanced_scene_render_matches_oracle(ctx, instanced, acc, shader):
    sc, states, blas_of, shading, _ = instanced
    cam = bt.Camera((-0.6, 0.6, -0.4, 0.4, 1, 100), (2, 3, -24), (-0.08, -0.12, 0.99), (0.99, 0, 0.08), (0, 1, 0))
    for lookup in (bt.LOOKUP_REFERENCE, bt.LOOKUP_HIT_OBJECT):
        rgba, ref = render_both(ctx, sc, states, blas_of, shading, cam, 200, 136, acc, shader, lookup)
        assert np.array_equal(rgba, ref), f"lookup {lookup}: {np.count_nonzero(rgba != ref)} bytes differ"
    assert len(np.unique(rgba.reshape(-1, 4), axis=0)) >= 2


def test_reference_lookup_outside_object_0_is_an_error_not_a_fault(ctx, instanced):
    """With object 0 on the smallest model, hits on larger models index past object 0's mesh: the
    reference panics there; the library reports BVHGPU_ERR_INVALID_ARG and the context stays usable."""
    _, states, _, shading, blases = instanced
    n = 6
    blas_of = np.array([2, 0, 1, 0, 1, 0], np.uint32)
    xf, inv = random_instances(n, 5, spread=3.0)
    sc = ctx.scene([blases[i] for i in blas_of], xf, inv)
    cam = bt.Camera((-1, 1, -1, 1, 1, 100), (0, 0, -12), (0, 0, 1), (1, 0, 0), (0, 1, 0))
    xf_d, inv_d = sc.download_transforms()
    tlas, used = sc.download_tlas()
    ref_tlas, ref_used, sa = checks.scene_state_reference(states, blas_of, xf_d, inv_d)
    with pytest.raises(orc.PanicError):
        orc.render_scene(cam.corners(), cam.view_inv, 64, 64, ref_tlas, sa, xf_d, bt.ACC_NORMAL, bt.SHADER_RADIANCE,
                         normals=[s[0] for s in shading], lookup=0)
    with pytest.raises(bt.BvhGpuError) as e:
        sc.render(cam, 64, 64, bt.ACC_NORMAL, bt.SHADER_RADIANCE, lookup=bt.LOOKUP_REFERENCE)
    assert e.value.code == 1
    # the same scene renders with the hit-object lookup, identical to the oracle
    rgba, _ = sc.render(cam, 64, 64, bt.ACC_NORMAL, bt.SHADER_RADIANCE, lookup=bt.LOOKUP_HIT_OBJECT)
    ref, _ = orc.render_scene(cam.corners(), cam.view_inv, 64, 64, ref_tlas, sa, xf_d, bt.ACC_NORMAL,
                              bt.SHADER_RADIANCE, normals=[s[0] for s in shading], lookup=1)
    assert np.array_equal(rgba, ref)
    sc.free()


def test_render_scene_rejects_bad_arguments(ctx, instanced):
    sc = instanced[0]
    cam = bt.Camera((-1, 1, -1, 1, 1, 100), (0, 0, -12), (0, 0, 1), (1, 0, 0), (0, 1, 0))
    for kwargs in ({"lookup": 2, "acc_params": ACC_PARAMS}, {"acc_params": None}):
        with pytest.raises(bt.BvhGpuError):
            sc.render(cam, 8, 8, bt.ACC_INTERSECTION, bt.SHADER_RADIANCE, **kwargs)
    with pytest.raises(bt.BvhGpuError):
        sc.render(cam, 8, 8, 7, bt.SHADER_RADIANCE)
