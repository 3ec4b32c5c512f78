"""Served relighting: incremental relight against a full bake with the
edited light table, and the relight server's results alone vs in a mix of
concurrent requests."""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _scene(ctx, seed, n_faces, k=128):
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    lit = scenes.lit_scene(seed, n_faces=n_faces, spacing=24.0, n_point=12, n_spot=3)
    env = Environment(ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    P = env.make_patches()
    env.make_transfers(scenes.transfer_directions(k))
    return lit, env, P["n_leaves"]


def _edits(descs, rng, n):
    """Move and rescale n of the point/spot lights in `descs` (scene light
    descriptions, updated in place); returns [(index, parsed light)]."""
    from dataclasses import replace

    from vrad_gb300.environment import make_light

    out = []
    idx = rng.choice(len(descs) - 1, size=n, replace=False)  # the last light is the sky
    for i in idx:
        li = descs[int(i)]
        o = tuple(float(c) for c in np.clip(np.asarray(li.origin) + rng.uniform(-300, 300, 3), 1, 4095))
        it = tuple(float(c) * float(rng.uniform(0.5, 2.0)) for c in li.intensity)
        descs[int(i)] = replace(li, origin=o, intensity=it)
        out.append((int(i), make_light(li.type, o, it, li.normal, **li.keys)))
    return out


def test_relight_equals_full_bake(gpu_ctx):
    lit, env, nl = _scene(gpu_ctx, 70, 80)
    env.relight_prepare(4, 5, 200, 1e-6)
    rng = np.random.default_rng(0)
    descs = list(lit.lights)
    for step in range(3):
        edits = _edits(descs, rng, 4)
        env.relight(edits, max_iters=200, rel_tol=1e-6)
        got = env.get_bake(nl)
        # a fresh scene baked from scratch with the edited table
        _, ref_env, _ = _scene(gpu_ctx, 70, 80)
        ref_env.set_lights(descs)
        ref_env.bake(4, 5, 200, 1e-6)
        ref = ref_env.get_bake(nl)
        assert np.array_equal(got["luxels"], ref["luxels"]), step
        assert np.array_equal(got["patch_direct"], ref["patch_direct"]), step
        scale = max(np.abs(ref["patch_total"]).max(), 1e-30)
        err = np.abs(got["patch_total"] - ref["patch_total"]) / np.maximum(
            np.abs(ref["patch_total"]), 1e-6 * scale)
        assert err.max() <= 1e-3, (step, err.max())


def test_server_same_alone_and_in_mix(gpu_ctx):
    from vrad_gb300.environment import Server

    def build():
        return [_scene(gpu_ctx, 80 + i, n) for i, n in enumerate([40, 96, 24])]

    rng = np.random.default_rng(1)
    descs = [list(lit.lights) for lit, _, _ in build()]
    plan = []
    for _ in range(24):
        s = int(rng.integers(0, 3))
        plan.append((s, _edits(descs[s], rng, int(rng.integers(1, 5)))))

    def run(slots, all_at_once):
        scenes = build()
        srv = Server(gpu_ctx, slots=slots, max_iters=32, rel_tol=1e-3)
        ids = []
        for lit, env, nl in scenes:
            env.relight_prepare(4, 9, 60, 1e-3)
            ids.append(srv.add_scene(env))
        tickets = []
        for s, edits in plan:
            t = srv.submit(ids[s], edits)
            if not all_at_once:
                assert srv.wait(t) == 0
            tickets.append(t)
        srv.drain()
        res = [srv.result(t) for t in tickets]
        finals = [env.get_bake(nl) for _, env, nl in scenes]
        srv.close()
        return res, finals

    alone, fa = run(1, False)
    mixed, fm = run(4, True)
    for a, m in zip(alone, mixed):
        assert a["status"] == m["status"] == 0
        assert a["bounces"] == m["bounces"] and a["delta"] == m["delta"]
        assert a["digest"] == m["digest"]
    for a, m in zip(fa, fm):
        assert np.array_equal(a["luxels"], m["luxels"])
        assert np.array_equal(a["patch_total"], m["patch_total"])
    # the mixed run really overlapped: some request started before an
    # earlier one (on another scene) had finished
    starts = sorted((m["start"], m["done"]) for m in mixed)
    assert any(starts[i + 1][0] < starts[i][1] for i in range(len(starts) - 1))


def test_sky_light_geometry_edit_rejected(gpu_ctx):
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import make_light

    lit, env, nl = _scene(gpu_ctx, 90, 12)
    env.relight_prepare(4, 0, 20, 1e-3)
    sky = len(lit.lights) - 1
    li = lit.lights[sky]
    ok = make_light(li.type, li.origin, (1.0, 2.0, 3.0))  # intensity only: allowed
    env.relight([(sky, ok)])
    bad = make_light(3, (0, 0, 0), (1.0, 1.0, 1.0), (0.0, 0.0, -1.0))  # turns into a sun
    with pytest.raises(VrgError, match="unsupported"):
        env.relight([(sky, bad)])


def test_admission_refuses_when_reserve_cannot_be_kept(gpu_ctx):
    # admission keeps the context's HBM reserve free: asking for more than the
    # GPU has turns the scene away with VRG_ERR_NOMEM, and the scene is
    # admitted once the reserve is back to normal
    from vrad_gb300._lib import VrgError

    lit, env, nl = _scene(gpu_ctx, 91, 24)
    gpu_ctx.set_hbm_reserve(1 << 60)
    try:
        with pytest.raises(VrgError, match="out of memory"):
            env.relight_prepare(4, 1, 20, 1e-3)
        with pytest.raises(VrgError, match="call out of order"):
            env.relight([], max_iters=4, rel_tol=1e-3)
    finally:
        gpu_ctx.set_hbm_reserve(1 << 30)
    env.relight_prepare(4, 1, 20, 1e-3)
    env.relight([], max_iters=4, rel_tol=1e-3)
