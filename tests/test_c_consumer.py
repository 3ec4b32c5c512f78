"""A plain C program linked against libvradgpu.so through include/vradgpu.h
(what a cgo or C caller does), run on the host: a host-only context builds a
scene and its trees, and the host entry points answer as documented."""
import shutil
import subprocess
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent

PROGRAM = r"""
#include <stdio.h>
#include "vradgpu.h"

#define CHECK(x) do { int rc_ = (x); if (rc_ != VRG_OK) { printf("FAIL %s = %d\n", #x, rc_); return 1; } } while (0)

int main(void) {
    vrg_ctx *ctx = NULL;
    vrg_env *env = NULL;
    CHECK(vrg_ctx_create(-1, &ctx));
    CHECK(vrg_env_create(ctx, &env));
    const float mn[3] = {0, 0, 0}, mx[3] = {64, 32, 16};
    CHECK(vrg_env_add_axis_aligned_rectangular_solid(env, VRG_TRACE_ID_OPAQUE, mn, mx, NULL));
    if (vrg_env_num_triangles(env) != 12) { printf("FAIL triangles\n"); return 1; }
    CHECK(vrg_env_setup_acceleration_structure(env));
    int64_t nodes = 0, refs = 0;
    int32_t height = 0;
    CHECK(vrg_env_tree_info(env, &nodes, &refs, &height));
    if (nodes < 1 || refs < 12) { printf("FAIL tree %lld %lld\n", (long long)nodes, (long long)refs); return 1; }
    /* device work on a host-only context is refused, not run on the CPU */
    const float a[3] = {1, 1, 1}, b[3] = {2, 2, 2};
    float frac = -1.0f;
    if (vrg_env_test_line_does_hit_sky(env, a, b, 1, -1, &frac) != VRG_ERR_STATE) { printf("FAIL state\n"); return 1; }
    const float verts[12] = {0, 0, 0, 64, 0, 0, 64, 64, 0, 0, 64, 0};
    const float vecs[8] = {1.0f / 16, 0, 0, 0, 0, 1.0f / 16, 0, 0};
    int32_t emin[2], esize[2], big = -1;
    CHECK(vrg_calc_face_extents(verts, 4, vecs, emin, esize, &big));
    if (emin[0] != 0 || esize[0] != 4 || esize[1] != 4 || big != 0) { printf("FAIL extents\n"); return 1; }
    vrg_bsp *bsp = NULL;
    const uint8_t junk[8] = {'X', 'B', 'S', 'P', 20, 0, 0, 0};
    if (vrg_bsp_open(junk, sizeof junk, &bsp) != VRG_ERR_INVALID || bsp != NULL) { printf("FAIL bsp\n"); return 1; }
    vrg_env_destroy(env);
    vrg_ctx_destroy(ctx);
    printf("OK\n");
    return 0;
}
"""


def test_c_program_uses_the_library(vlib, tmp_path):
    from vrad_gb300 import build

    cc = shutil.which("gcc") or shutil.which("cc")
    if cc is None:
        pytest.skip("no C compiler")
    src = tmp_path / "use.c"
    src.write_text(PROGRAM)
    exe = tmp_path / "use"
    lib_dir = build.LIB.parent
    r = subprocess.run([cc, "-std=c11", "-Wall", "-Werror", "-I", str(ROOT / "include"), str(src),
                        "-o", str(exe), "-L", str(lib_dir), "-lvradgpu",
                        f"-Wl,-rpath,{lib_dir}"], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    run = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120)
    assert run.returncode == 0 and run.stdout.strip() == "OK", run.stdout + run.stderr
