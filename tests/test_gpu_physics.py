"""Physics-driven instance transforms (Scene::run: World::run_physics, SceneObject::update_transform,
Tlas::rebuild) on the device against the oracle's restatement of BT/src/physics/.

Bit for bit in the reference demos' setting (drag 1, can_sleep false -- powf is never reached)
with gravity and springs, over 60 steps, directly and replayed from a CUDA graph: the bodies,
the object transforms and inverses, the TLAS and the traced hits.  With drag < 1 and sleeping
bodies powf enters (its last bit is the math library's), so those runs are checked within a
relative 1e-5."""
import numpy as np
import pytest

import bvhtracer_gb300 as bt
from bvhtracer_gb300 import scenes
from oracle import oracle as orc

pytestmark = pytest.mark.gpu
DT = np.float32(1.0 / 30.0)


def world_setup(n, seed, demo=True):
    rng = np.random.default_rng(seed)
    bodies = bt.rigid_body_default(n)
    bodies["inverse_mass"] = rng.uniform(0.2, 2.0, n)
    inertia = rng.uniform(0.5, 2.0, (n, 3))
    for i in range(n):
        bodies[i]["inverse_inertia"] = np.diag(1.0 / inertia[i]).astype(np.float32).reshape(9)
    bodies["position"] = rng.uniform(-8, 8, (n, 3))
    q = rng.standard_normal((n, 4))
    bodies["orientation"] = (q / np.linalg.norm(q, axis=1, keepdims=True)).astype(np.float32)
    bodies["rotation"] = rng.uniform(-1, 1, (n, 3))
    bodies["velocity"] = rng.uniform(-0.5, 0.5, (n, 3))
    bodies["is_awake"] = 1
    if demo:
        bodies["can_sleep"] = 0
    else:
        bodies["can_sleep"] = np.arange(n) % 2
        bodies["linear_drag"] = 0.9
        bodies["angular_drag"] = 0.8
    gens = np.zeros(n + n // 2, bt.FORCE_GENERATOR)
    for i in range(n):  # gravity on every body (registered first), then springs between pairs
        gens[i]["kind"] = bt.FORCE_GRAVITY
        gens[i]["body"] = i
        gens[i]["gravity"] = (0.0, -9.8 if i % 3 else -1.5, 0.0)
    for k in range(n // 2):
        g = gens[n + k]
        g["kind"] = bt.FORCE_SPRING
        g["body"] = 2 * k
        g["other"] = 2 * k + 1
        g["spring_point"] = rng.uniform(-0.5, 0.5, 3)
        g["other_point"] = rng.uniform(-0.5, 0.5, 3)
        g["spring_constant"] = rng.uniform(1, 5)
        g["rest_length"] = rng.uniform(1, 3)
    return bodies, gens


def scale_translate(n, seed):
    rng = np.random.default_rng(seed)
    init = np.zeros((n, 16), np.float32)
    for i in range(n):
        m = np.eye(4, dtype=np.float32) * np.float32(rng.uniform(0.5, 1.5))
        m[3, 3] = 1
        m[3, :3] = rng.uniform(-1, 1, 3)  # column-major: translation in column 3
        init[i] = m.reshape(16)
    return init


@pytest.mark.parametrize("graph", [False, True])
def test_scene_run_matches_the_oracle_bit_for_bit(graph):
    n = 16
    bodies, gens = world_setup(n, 3)
    init = scale_translate(n, 4)
    tris, bvh = None, None
    with bt.Context(0) as ctx:
        tris = scenes.displaced_icosphere(3, 5).triangles().copy()
        bvh = bt.BvhBuilder().build_for(tris)
        blas = ctx.upload_blas(bvh, tris)
        ref_bodies = bodies.copy()
        orc.world_start_frame(ref_bodies)
        world = ctx.world(bodies)
        world.start_frame_async()
        w2 = ctx.world(ref_bodies)  # placeholder world to exercise create/free
        w2.free()
        world.free()
        world = ctx.world(bodies, gens)
        world.start_frame_async()
        body_of = np.arange(n, dtype=np.uint32)
        xf0, inv0 = orc.object_transforms(ref_bodies, body_of, init)
        sc = ctx.scene([blas] * n, xf0, inv0)
        sc.bind_world(world, body_of, init)
        steps = 60
        if graph:
            ctx.graph_begin()
            sc.run_async(float(DT))
            gid = ctx.graph_end()
            for _ in range(steps):
                ctx.graph_launch(gid)
        else:
            for _ in range(steps):
                sc.run_async(float(DT))
        ctx.sync()
        got = world.download()
        for _ in range(steps):
            orc.world_step(ref_bodies, gens, DT)
        assert got.tobytes() == ref_bodies.tobytes(), "rigid bodies differ"
        xf, inv = sc.download_transforms()
        rxf, rinv = orc.object_transforms(ref_bodies, body_of, init)
        assert xf.tobytes() == rxf.tobytes() and inv.tobytes() == rinv.tobytes()
        tlas, tused = sc.download_tlas()
        root = bvh.nodes[0]
        omin = np.zeros((n, 3), np.float32)
        omax = np.zeros((n, 3), np.float32)
        for i in range(n):
            omin[i], omax[i] = orc.object_bounds(root["bounds_min"], root["bounds_max"], rxf[i])
        ref_tlas, ref_used = orc.tlas_build(omin, omax)
        assert tused == ref_used and tlas.tobytes() == ref_tlas.tobytes()
        rays = scenes.sphere_rays(20000, 8, box=30.0)
        sa = orc.SceneArrays([(bvh.nodes[:bvh.nodes_used], bvh.nodes_used, tris)], np.zeros(n, np.int64), rinv)
        ref = orc.scene_intersect(ref_tlas, ref_used, sa, rays)
        assert sc.intersect(rays).tobytes() == ref.tobytes()
        moved = np.abs(got["position"] - bodies["position"]).max()
        assert moved > 1.0  # the bodies fell and swung


def test_drag_and_sleep_within_tolerance():
    n = 12
    bodies, gens = world_setup(n, 9, demo=False)
    ref = bodies.copy()
    with bt.Context(0) as ctx:
        world = ctx.world(bodies, gens)
        world.start_frame_async()
        for _ in range(45):
            world.step_async(float(DT))
        got = world.download()
    orc.world_start_frame(ref)
    for _ in range(45):
        orc.world_step(ref, gens, DT)
    for f in ("position", "velocity", "orientation", "transform"):
        a, b = got[f].astype(np.float64), ref[f].astype(np.float64)
        assert np.all(np.abs(a - b) <= 1e-5 * np.maximum(np.abs(b), 1.0)), f
    assert np.array_equal(got["is_awake"], ref["is_awake"])
