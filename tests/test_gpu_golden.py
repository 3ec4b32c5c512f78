"""The C-ABI path on the GPU against the committed golden fixtures: shadow
lines and rays decided by float64 geometry (bit-exact hit indices and
occlusion bits), and a small lit scene's luxels (1e-4 relative), transfer CSR
(identical), patch direct light (1e-4) and bounce (1e-3 of float64)."""
import numpy as np
import pytest

from test_golden import check_against_geometry, geom, mg, pipe  # noqa: F401

pytestmark = pytest.mark.gpu

RTOL_DIRECT = 1e-4
RTOL_BOUNCE = 1e-3


def _rel_err(a, b, floor):
    a = a.astype(np.float64)
    b = b.astype(np.float64)
    return np.abs(a - b) / np.maximum(np.abs(b), floor * max(np.abs(b).max(), 1e-30))


@pytest.fixture(scope="module")
def geom_env(gpu_ctx, geom):
    from vrad_gb300.environment import Environment

    env = Environment(gpu_ctx)
    env.add_triangles(geom["xyz"], geom["ids"])
    env.SetupAccelerationStructure()
    return env


@pytest.mark.parametrize("k", [0, 1])
def test_lines_match_float64_geometry(geom_env, geom, k):
    g = geom
    skip = int(g["skip_ids"][k])
    mask, hit, t = geom_env.occlusion_mask(g["starts"], g["stops"], skip_id=skip, closest=True)
    check_against_geometry(g, k, hit, t, mask=mask)
    # testline.go:36 skips id TRACE_ID_STATICPROP | staticPropToSkip
    prop = -1 if skip == -1 else skip & ~mg.scenes.TRACE_ID_STATICPROP
    frac = geom_env.test_line_does_hit_sky(g["starts"], g["stops"], prop)
    check_against_geometry(g, k, hit, t, frac=frac)
    # the same segments as rays (unit direction, [0, len))
    d = (g["stops"] - g["starts"]).astype(np.float32)
    ln = np.sqrt((d[:, 0] * d[:, 0] + d[:, 1] * d[:, 1]) + d[:, 2] * d[:, 2])
    dn = d * (np.float32(1.0) / ln)[:, None]
    rhit, rt = geom_env.trace_closest(g["starts"], dn, 0.0, ln, skip)
    check_against_geometry(g, k, rhit, rt)


def test_pipeline_matches_fixture(gpu_ctx, pipe):
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    lit = mg.pipeline_scene()
    assert mg.pipeline_inputs_digest(lit) == str(pipe["inputs"])
    env = Environment(gpu_ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    rgb, rays = env.gather_direct_light(supersamples=mg.PIPE["ss"], seed=mg.PIPE["gather_seed"])
    assert rays == int(pipe["rays"])
    assert _rel_err(rgb, pipe["luxel_rgb"], 1e-3).max() <= RTOL_DIRECT

    P = env.make_patches()
    assert mg.patch_digest(P) == str(pipe["patches"])
    nl = P["n_leaves"]
    k = mg.PIPE["k"]
    nnz = env.make_transfers(scenes.transfer_directions(k))
    row_ptr, col, w = env.get_transfers(nl, nnz)
    cnt = np.rint(w.astype(np.float64) * k).astype(np.int32)
    assert np.array_equal(cnt.astype(np.float32) / np.float32(k), w)
    assert mg.sha(row_ptr, col, cnt) == str(pipe["transfers"])

    direct = env.gather_patch_direct(nl)
    assert _rel_err(direct, pipe["patch_direct"], 1e-6).max() <= RTOL_DIRECT
    total, iters, _ = env.bounce_light(nl, max_bounces=100, rel_tol=1e-3)
    assert iters == int(pipe["bounce_iters"])
    assert _rel_err(total, pipe["bounce_total"], 1e-6).max() <= RTOL_BOUNCE
