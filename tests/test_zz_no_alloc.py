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
        # the context set the array up, so no call allocates, the first included
        assert torch.cuda.mem_get_info()[0] == free_before
        got = out[:, :3].cpu().numpy()
        # The per-row sums are the same as the allocating path's; only the
        # double-precision energy sums that decide when to stop are added in
        # another block order.  A count one apart is accepted only when the
        # allocating path's last delta sits on the tolerance.
        if b.value != ref_b:
            assert abs(b.value - ref_b) == 1 and abs(ref_d - 1e-3) <= 1e-9, (b.value, ref_b, ref_d)
            continue
        scale = max(np.abs(ref).max(), 1e-30)
        err = np.abs(got - ref) / np.maximum(np.abs(ref), 1e-6 * scale)
        assert err.max() <= BOUNCE_RTOL, (call, err.max())
        assert abs(d.value - ref_d) <= BOUNCE_RTOL * max(abs(ref_d), 1e-12)


def test_noalloc_bounce_refuses_bad_output_before_launching(scene):
    # A host pointer or a device pointer off the 16-byte grid would fault on
    # the GPU; the call refuses both up front and launches nothing.
    import torch

    env, nl = scene
    host = np.zeros((nl, 4), np.float32)
    dev = torch.empty((nl + 1, 4), dtype=torch.float32, device="cuda")
    launches = env.ctx.launch_count()
    for ptr in (host.ctypes.data, dev.data_ptr() + 4):
        rc = env.lib.vrg_env_bounce_light_noalloc(env.h, 10, C.c_float(1e-3), C.c_void_p(ptr),
                                                  None, None)
        assert rc == -1, rc  # VRG_ERR_INVALID
    assert env.ctx.launch_count() == launches
