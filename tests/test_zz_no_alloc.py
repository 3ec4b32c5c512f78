"""vrg_env_bounce_light_noalloc: the bounce loop for callers that may not
allocate device memory while they run (for example a serving loop that
reserved its memory up front, or a process whose memory belongs to a
framework pool).  Its working state sits in one fixed device array inside
the library, so the call allocates nothing.

The test calls it through the C ABI twice in a row and compares each result
with the allocating entry point (vrg_env_bounce_light) on the same resident
scene, within the bounce tolerance the other tests use.  This file is named
so pytest collects it last."""
import ctypes as C

import numpy as np
import pytest

from conftest import small_lit_scene

pytestmark = pytest.mark.gpu

BOUNCE_RTOL = 1e-3


@pytest.fixture(scope="module")
def scene(gpu_ctx):
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    lit = small_lit_scene(160, seed=21)
    env = Environment(gpu_ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    P = env.make_patches()
    env.make_transfers(scenes.transfer_directions(256))
    env.gather_patch_direct(P["n_leaves"])
    return env, P["n_leaves"]


def test_noalloc_bounce_matches_allocating_bounce_twice(scene):
    import torch

    env, nl = scene
    ref, ref_b, ref_d = env.bounce_light(nl, max_bounces=60, rel_tol=1e-3)
    assert ref_b > 1 and np.abs(ref).max() > 0
    out = torch.empty((nl, 4), dtype=torch.float32, device="cuda")
    for call in range(2):
        out.fill_(float("nan"))  # every call must overwrite the whole output
        torch.cuda.synchronize()
        free_before = torch.cuda.mem_get_info()[0]
        b = C.c_int32()
        d = C.c_float()
        rc = env.lib.vrg_env_bounce_light_noalloc(env.h, 60, C.c_float(1e-3),
                                                  C.c_void_p(out.data_ptr()), C.byref(b),
                                                  C.byref(d))
        assert rc == 0, env.lib.vrg_last_error(env.ctx.h)
        torch.cuda.synchronize()
        if call == 1:
            assert torch.cuda.mem_get_info()[0] == free_before
        got = out[:, :3].cpu().numpy()
        assert b.value == ref_b
        scale = max(np.abs(ref).max(), 1e-30)
        err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-6 * scale)
        assert err.max() <= BOUNCE_RTOL, (call, err.max())
        assert abs(d.value - ref_d) <= BOUNCE_RTOL * max(abs(ref_d), 1e-12)
