"""Parity at the benchmark's own sizes.

- The direct-light gather of the 4,096-face scene (1,329,508 luxels x 4
  samples, 72 lights + the 162-direction sky): every luxel against the
  oracle, relative error <= 1e-4 with no absolute floor.
- Transfers of the same faces subdivided at 64 units (142,524 leaf patches)
  at 65,536 rays per patch (about 2,000 entries per row): 1,000 seeded rows,
  plus every row that overflowed the shared-memory row table, rebuilt by the
  oracle and compared bit for bit with the device CSR.
- The bounce over that full CSR (downloaded) against the float64 oracle:
  bounced light within 1e-3 relative, the same bounce count.
Each test prints its error figures."""
import os

import numpy as np
import pytest

from conftest import rel_error_stats

pytestmark = pytest.mark.gpu

THREADS = os.cpu_count() or 8
RTOL_DIRECT = 1e-4
RTOL_BOUNCE = 1e-3
K_CONFIG2 = 65536


def test_direct_full_config_every_luxel(gpu_ctx, lit_scene, oracle):
    from vrad_gb300.environment import Environment

    env = Environment(gpu_ctx)
    env.add_triangles(lit_scene.xyz, lit_scene.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit_scene)
    env.set_lights(lit_scene.lights)
    rgb, rays = env.gather_direct_light(supersamples=4, seed=0)
    s = oracle.Scene(lit_scene.xyz, lit_scene.ids)
    ref, rrays = oracle.gather_luxels(s, oracle.make_lights(lit_scene.lights), len(lit_scene.lights),
                                      lit_scene, 0, lit_scene.n_faces, ss=4, seed=0, threads=THREADS)
    st = rel_error_stats(rgb, ref)
    print("direct, 4096 faces:", st, "rays", rays)
    assert rays == rrays
    assert st["zero_ref_nonzero"] == 0
    assert st["max_rel"] <= RTOL_DIRECT, st


@pytest.fixture(scope="module")
def config2(gpu_ctx, lit_scene, oracle):
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    env = Environment(gpu_ctx)
    env.add_triangles(lit_scene.xyz, lit_scene.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit_scene)
    env.set_lights(lit_scene.lights)
    P = env.make_patches()
    nl = P["n_leaves"]
    dirs = scenes.transfer_directions(K_CONFIG2)
    nnz = env.make_transfers(dirs)
    k, nnz2, ovf = env.transfer_info()
    assert (k, nnz2) == (K_CONFIG2, nnz)
    row_ptr, col, w = env.get_transfers(nl, nnz)
    OP = oracle.make_patches(lit_scene)
    return dict(env=env, P=P, nl=nl, dirs=dirs, nnz=nnz, ovf=ovf, row_ptr=row_ptr, col=col, w=w,
                OP=OP, s=oracle.Scene(lit_scene.xyz, lit_scene.ids))


def test_transfers_config2_sampled_rows(config2, lit_scene, oracle):
    c = config2
    nl, row_ptr = c["nl"], c["row_ptr"]
    per_row = np.diff(row_ptr)
    print(f"config-2 CSR: {nl} rows, {c['nnz']} entries, {c['nnz'] / nl:.1f} per row, "
          f"max {per_row.max()}, {c['ovf']} rows past the row table")
    assert c["nnz"] / nl > 1800  # the config's ~2,000 weights per patch
    rng = np.random.default_rng(20)
    rows = set(rng.choice(nl, 1000, replace=False).tolist())
    rows |= set(np.nonzero(per_row > 7168)[0].tolist())  # the overflow path's rows
    rows = np.array(sorted(rows), np.int64)
    orow, ocol, ocnt = oracle.make_transfer_rows(c["s"], lit_scene, c["OP"], c["dirs"], rows,
                                                 threads=THREADS)
    k = np.float32(K_CONFIG2)
    mism = 0
    for j, r in enumerate(rows):
        a, b = row_ptr[r], row_ptr[r + 1]
        oa, ob = orow[j], orow[j + 1]
        same = (b - a == ob - oa and np.array_equal(c["col"][a:b], ocol[oa:ob]) and
                np.array_equal(c["w"][a:b].view(np.uint32),
                               (ocnt[oa:ob] / k).astype(np.float32).view(np.uint32)))
        mism += not same
    print(f"sampled rows: {len(rows)}, mismatching rows: {mism}")
    assert mism == 0


def test_bounce_config2_vs_float64(config2, lit_scene, oracle):
    c = config2
    env, nl, OP = c["env"], c["nl"], c["OP"]
    direct = env.gather_patch_direct(nl)
    leaf_patch = np.nonzero(OP["leaf_index"] >= 0)[0]
    face = OP["face"][leaf_patch]
    pts = (OP["center"][leaf_patch] + lit_scene.normal[face] * np.float32(0.125)).astype(np.float32)
    ref_direct, _ = oracle.gather_points(c["s"], oracle.make_lights(lit_scene.lights),
                                         len(lit_scene.lights), pts, lit_scene.normal[face],
                                         threads=THREADS)
    sd = rel_error_stats(direct, ref_direct)
    print("leaf-patch direct light:", sd)
    assert sd["zero_ref_nonzero"] == 0 and sd["max_rel"] <= RTOL_DIRECT
    total, b, delta = env.bounce_light(nl, max_bounces=100, rel_tol=1e-3)
    refl = lit_scene.refl[face]
    rtot, rb, rdeltas = oracle.bounce_f64(c["row_ptr"], c["col"], c["w"], refl, ref_direct,
                                          np.zeros_like(refl), 100, 1e-3, threads=THREADS)
    nz = rtot != 0
    rel = np.abs(total.astype(np.float64)[nz] - rtot[nz]) / np.abs(rtot[nz])
    print(f"bounce: {b} bounces (oracle {rb}), delta {delta:.4g} (oracle {rdeltas[-1]:.4g}), "
          f"max rel {rel.max():.3g}, p99 rel {np.percentile(rel, 99):.3g}")
    assert b == rb
    assert np.all(total[~nz] == 0)
    assert rel.max() <= RTOL_BOUNCE
