"""Autotuned launch sites: every variant gives the same bits, the first
launch in a bucket records a choice with one time per variant, and a saved
choice loads back."""
import numpy as np
import pytest

from conftest import bits_equal, small_lit_scene


def _force(ctx, tmp_path, key, variant):
    p = tmp_path / f"tune_{variant}.txt"
    p.write_text(f"{key} {variant}\n")
    ctx.autotune_load(str(p))
    assert ctx.autotune_choice(key)[0] == variant


def test_tune_file_round_trip_host(host_ctx, tmp_path):
    from vrad_gb300.environment import Context

    key = Context.tune_key("trace_mask", 12300, 1 << 20)
    assert key == "trace_mask/t13/n20"
    assert Context.tune_key("direct_luxels", 1, 0) == "direct_luxels/t0/n0"
    assert host_ctx.autotune_choice("nope/t1/n1")[0] == -1
    _force(host_ctx, tmp_path, key, 2)
    out = tmp_path / "saved.txt"
    host_ctx.autotune_save(str(out))
    assert f"{key} 2" in out.read_text().splitlines()
    # out-of-range variants in a file are ignored (a site has at most 32)
    bad = tmp_path / "bad.txt"
    bad.write_text("trace_mask/t1/n1 99\ntrace_mask/t2/n2 32\ntrace_mask/t3/n3 -1\n")
    host_ctx.autotune_load(str(bad))
    for k in ("trace_mask/t1/n1", "trace_mask/t2/n2", "trace_mask/t3/n3"):
        assert host_ctx.autotune_choice(k)[0] == -1
    _force(host_ctx, tmp_path, "trace_mask/t4/n4", 31)


@pytest.mark.gpu
def test_trace_mask_variants_identical(gpu_ctx, anyhit_scene, tmp_path):
    from vrad_gb300.environment import Context, Environment

    sc = anyhit_scene
    env = Environment(gpu_ctx)
    env.add_triangles(sc.xyz, sc.ids)
    env.SetupAccelerationStructure()
    # all 2^20 lines: a variant whose arithmetic differed in a rare case
    # (one line in millions) would pass on a few thousand
    n = sc.starts.shape[0]
    a, b = sc.starts, sc.stops
    for closest in (False, True):
        key = Context.tune_key("trace_mask_hit" if closest else "trace_mask", env.num_triangles(), n)
        outs = []
        for v in range(20):
            _force(gpu_ctx, tmp_path, key, v)
            outs.append(env.occlusion_mask(a, b, closest=closest))
        for o in outs[1:]:
            if closest:
                assert all(bits_equal(x, y) for x, y in zip(o, outs[0]))
            else:
                assert np.array_equal(o, outs[0])


@pytest.mark.gpu
def test_direct_variants_identical_and_choice_recorded(gpu_ctx, tmp_path):
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Context, Environment

    lit = scenes.lit_scene(0)  # the full 4,096-face workload, 5.3M samples
    env = Environment(gpu_ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    key = Context.tune_key("direct_luxels", env.num_triangles(), env.num_luxels() * 4)
    assert gpu_ctx.autotune_choice(key)[0] == -1
    rgb0, rays0 = env.gather_direct_light(supersamples=4, seed=2)  # tunes this bucket
    v, ms = gpu_ctx.autotune_choice(key)
    assert v in range(12) and len(ms) == 12
    for v in range(12):
        _force(gpu_ctx, tmp_path, key, v)
        rgb, rays = env.gather_direct_light(supersamples=4, seed=2)
        assert rays == rays0
        assert bits_equal(rgb, rgb0)


@pytest.mark.gpu
def test_transfer_variants_identical(gpu_ctx, tmp_path):
    # every row-kernel variant gives the same CSR (columns, weights, row
    # starts) on the full 4,096-face scene at K = 2,048
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Context, Environment

    lit = scenes.lit_scene(0)
    env = Environment(gpu_ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    nl = env.make_patches()["n_leaves"]
    k = 2048
    dirs = scenes.transfer_directions(k)
    key = Context.tune_key("transfer_rows", env.num_triangles(), nl * k)
    ref = None
    for v in range(6):
        _force(gpu_ctx, tmp_path, key, v)
        nnz = env.make_transfers(dirs)
        got = env.get_transfers(nl, nnz)
        if ref is None:
            ref = got
            continue
        assert np.array_equal(got[0], ref[0]) and np.array_equal(got[1], ref[1])
        assert bits_equal(got[2], ref[2])


@pytest.mark.gpu
def test_bounce_variants_identical(gpu_ctx, tmp_path):
    # 4, 8 or 2 entries per lane per round sum the same entries in the same
    # order with fused multiply-adds: identical totals
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Context, Environment

    lit = small_lit_scene(240, seed=4)
    env = Environment(gpu_ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    nl = env.make_patches()["n_leaves"]
    nnz = env.make_transfers(scenes.transfer_directions(1024))
    env.gather_patch_direct(nl)
    key = Context.tune_key("bounce_spmv", nnz, nl)
    outs = []
    for v in range(7):
        _force(gpu_ctx, tmp_path, key, v)
        total, bounces, _ = env.bounce_light(nl, max_bounces=12, rel_tol=0.0)
        assert bounces == 12
        outs.append(total)
    assert np.abs(outs[0]).max() > 0
    for o in outs[1:]:
        assert bits_equal(o, outs[0])
