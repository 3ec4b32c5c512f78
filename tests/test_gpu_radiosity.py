"""GPU parity of transfer building (CSR identical to the oracle's: it is
built from bit-exact closest hits) and of the bounce loop (within 1e-3
relative of the float64 oracle)."""
import numpy as np
import pytest

from conftest import small_lit_scene

pytestmark = pytest.mark.gpu

BOUNCE_RTOL = 1e-3


@pytest.fixture(scope="module")
def radiosity(gpu_ctx, oracle):
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    lit = small_lit_scene(192, seed=9)
    env = Environment(gpu_ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    P = env.make_patches()
    k = 512
    dirs = scenes.transfer_directions(k)
    nnz = env.make_transfers(dirs)
    row_ptr, col, w = env.get_transfers(P["n_leaves"], nnz)
    s = oracle.Scene(lit.xyz, lit.ids)
    OP = oracle.make_patches(lit)
    orow, ocol, ocnt = oracle.make_transfers(s, lit, OP, dirs, threads=16)
    return dict(lit=lit, env=env, P=P, k=k, row_ptr=row_ptr, col=col, w=w, orow=orow, ocol=ocol,
                ocnt=ocnt, s=s, OP=OP)


def test_transfers_csr_identical(radiosity):
    r = radiosity
    assert np.array_equal(r["row_ptr"], r["orow"])
    assert np.array_equal(r["col"], r["ocol"])
    assert np.array_equal(r["w"], (r["ocnt"] / np.float32(r["k"])).astype(np.float32))
    # rows sorted, unique, weights in (0, 1], row sums <= 1
    rp, col = r["row_ptr"], r["col"]
    for i in range(len(rp) - 1):
        c = col[rp[i]:rp[i + 1]]
        assert (np.diff(c) > 0).all()
    sums = np.add.reduceat(r["w"], rp[:-1])[np.diff(rp) > 0]
    assert (sums <= 1.0 + 1e-6).all()


def test_patch_direct_and_bounce_vs_float64(radiosity, oracle):
    r = radiosity
    lit, env, OP = r["lit"], r["env"], r["OP"]
    nl = r["P"]["n_leaves"]
    direct = env.gather_patch_direct(nl)
    leaf_patch = np.nonzero(OP["leaf_index"] >= 0)[0]
    face = OP["face"][leaf_patch]
    pts = (OP["center"][leaf_patch] + lit.normal[face] * np.float32(0.125)).astype(np.float32)
    ref_direct, _ = oracle.gather_points(r["s"], oracle.make_lights(lit.lights), len(lit.lights),
                                         pts, lit.normal[face], threads=16)
    np.testing.assert_allclose(direct, ref_direct, rtol=1e-4, atol=1e-6 * ref_direct.max())
    refl = lit.refl[face]
    base = np.zeros_like(refl)
    w64 = (r["ocnt"] / np.float32(r["k"])).astype(np.float32)
    for max_b, tol in ((6, 0.0), (100, 1e-3)):
        total, b, delta = env.bounce_light(nl, max_bounces=max_b, rel_tol=tol)
        rtot, rb, rdeltas = oracle.bounce_f64(r["orow"], r["ocol"], w64, refl, ref_direct, base,
                                              max_b, tol)
        assert b == rb, (b, rb)
        abs_tol = 1e-6 * np.abs(rtot).max()
        err = np.abs(total - rtot) / np.maximum(np.abs(rtot), abs_tol)
        assert err.max() <= BOUNCE_RTOL, err.max()
        assert abs(delta - rdeltas[-1]) <= 1e-3 * rdeltas[-1] + 1e-9


def test_bounce_repeatable(radiosity):
    r = radiosity
    nl = r["P"]["n_leaves"]
    t1, b1, _ = r["env"].bounce_light(nl, 20, 1e-3)
    t2, b2, _ = r["env"].bounce_light(nl, 20, 1e-3)
    assert b1 == b2 and np.array_equal(t1, t2)


def test_transfers_overflow_path_identical(gpu_ctx, radiosity):
    # a low table limit sends most rows to the global-memory sort; the CSR
    # must not change
    from vrad_gb300 import scenes

    r = radiosity
    env = r["env"]
    try:
        gpu_ctx.set_transfer_table_limit(16)
        nnz = env.make_transfers(scenes.transfer_directions(r["k"]))
        k, nnz2, ovf = env.transfer_info()
        assert (k, nnz2) == (r["k"], nnz) and ovf > 0
        row_ptr, col, w = env.get_transfers(r["P"]["n_leaves"], nnz)
    finally:
        gpu_ctx.set_transfer_table_limit(7168)
        env.make_transfers(scenes.transfer_directions(r["k"]))
    assert np.array_equal(row_ptr, r["orow"])
    assert np.array_equal(col, r["ocol"])
    assert np.array_equal(w, (r["ocnt"] / np.float32(r["k"])).astype(np.float32))
    assert env.transfer_info()[2] == 0
