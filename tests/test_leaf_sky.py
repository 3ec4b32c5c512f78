"""CanLeafTraceToSky's lines (rad/lightmap/lightmap.go:425-451) on the CPU:
the library's line generator against a numpy restatement over the 162
directions of the generated table; the device entry point is refused on a
host-only context."""
import re
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent


def anorms():
    text = (ROOT / "vrad_gb300" / "csrc" / "anorms_table.h").read_text()
    body = text[text.index("VRG_ANORMS_INIT"):]
    vals = re.findall(r"[-+]?\d+\.\d+(?:[eE][-+]?\d+)?f?", body)
    a = np.array([float(v.rstrip("f")) for v in vals], np.float32)
    assert a.size == 162 * 3
    return a.reshape(162, 3)


def test_leaf_sky_lines_match_numpy(vlib):
    from vrad_gb300.environment import leaf_sky_lines

    rng = np.random.default_rng(6)
    mins = rng.integers(-16384, 16000, (50, 3)).astype(np.int32)
    maxs = (mins + rng.integers(1, 2000, (50, 3))).astype(np.int32)
    mins[0], maxs[0] = (-16384, -16384, -16384), (16384, 16384, 16384)  # sums past int16
    a, b = leaf_sky_lines(mins, maxs)
    centre = (mins + maxs).astype(np.float32) * np.float32(0.5)
    L = np.float32(1.732050807569 * 32768.0)
    want_b = (anorms()[None, :, :] * -L + centre[:, None, :]).reshape(-1, 3)
    assert np.array_equal(a, np.repeat(centre, 162, axis=0))
    assert np.array_equal(b, want_b)


def test_leaf_sky_needs_a_device(vlib, host_ctx):
    from vrad_gb300._lib import VrgError
    from vrad_gb300.environment import Environment

    env = Environment(host_ctx)
    env.add_triangles(np.zeros((1, 9), np.float32), np.zeros(1, np.int32))
    env.SetupAccelerationStructure()
    with pytest.raises(VrgError):
        env.CanLeafTraceToSky([[0, 0, 0]], [[1, 1, 1]])
