"""Benchmark of the radiosity hot path on GB300.

Headline (`value`): the direct-light pass of a bake (4,096 box faces, 1.33M
luxels x 4 supersamples, 64 point + 8 spot lights + a 162-direction sky,
8,208-triangle room whose ceiling is sky).  A step is one full gather; the
metric is shadow rays traced per second (Mrays/s), with the whole bake
compared luxel by luxel against the oracle (`parity`).

The same JSON line carries the rest of the metric, one object per workload,
each with its own error against the oracle and its roofline:
  anyhit     2^20 shadow lines, 12,300 triangles: mask and closest-hit Mrays/s
  rooms      the headline bake with the wall cells off, and with the room's
             walls split into 16 x 16 tiles per face: what the cells buy
  radiosity  the same faces at 64-unit patches, 65,536 transfer rays per
             patch: CSR build, bounce SpMV GB/s, solve to 1e-3
  batch      256 scenes baked together vs one scene per launch: bakes/s
  serve      8 resident scenes, Poisson relight requests: p50/p99 ms, bakes/s
`--headline-only` skips them; `--workload X` prints one of them as its own
line.

`--impl reference` times the reference's CPU path instead: the C
restatement of it under oracle/ (the Go reference has no toolchain here),
with every host thread, on a bounded sample per step.
"""
from __future__ import annotations

import argparse
import ctypes as C
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

SEED = 0
STATS_SAMPLE_FACES = 256  # faces whose walk is counted for the byte model
REF_FACES_PER_STEP = 256  # reference arm: faces per timed step


def _env_int(name, default):
    try:
        return int(os.environ.get(name, default))
    except ValueError:
        return default


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _profile_value(kernel_file: str, key: str):
    """A `key: value` figure from a committed ncu summary under profiles/."""
    p = ROOT / "profiles" / kernel_file
    if not p.exists():
        return None
    for line in p.read_text().splitlines():
        if line.startswith(key + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def _ncu_traffic(kernel_file: str):
    """DRAM bytes per launch from a committed ncu summary, if present."""
    return _profile_value(kernel_file, "dram_bytes_per_launch_full")


def rel_error_stats(got, ref, floor_frac=1e-3):
    """Error of a device result against the oracle: share of bit-identical
    values, max / p99 of |got - ref| / |ref| over ref != 0 (no floor), how
    many ref == 0 values the device did not give as 0, and how many values
    lie under floor_frac x max |ref| (counted, not excused)."""
    g = np.ascontiguousarray(got, dtype=np.float32).ravel()
    r = np.ascontiguousarray(ref, dtype=np.float32).ravel()
    g64, r64 = g.astype(np.float64), r.astype(np.float64)
    nz = r64 != 0.0
    rel = np.abs(g64[nz] - r64[nz]) / np.abs(r64[nz])
    top = float(np.abs(r64).max()) if r64.size else 0.0
    return {"values": int(g.size),
            "bit_identical": round(float(np.mean(g.view(np.uint32) == r.view(np.uint32))), 6),
            "max_rel": float(rel.max()) if rel.size else 0.0,
            "p99_rel": float(np.percentile(rel, 99)) if rel.size else 0.0,
            "zero_ref_nonzero": int(np.count_nonzero(g64[~nz])),
            f"under_{floor_frac:g}_of_max": int(np.count_nonzero(np.abs(r64) < floor_frac * top))}


def issue_roofline(inst_per_unit, units, kernel_ms, sm_mhz, sms, source):
    """Warp instructions issued per second against the SMs' issue rate (one
    warp instruction per scheduler per cycle, 4 schedulers per SM)."""
    if not inst_per_unit or not sm_mhz or not kernel_ms:
        return None
    achieved = inst_per_unit * units / (kernel_ms * 1e-3) / 1e9
    peak = sms * 4 * sm_mhz * 1e6 / 1e9
    return {"achieved": round(achieved, 1), "peak": round(peak, 1),
            "unit": "G warp instructions/s", "frac": round(achieved / peak, 4),
            "warp_instructions_per_unit": inst_per_unit, "sm_mhz": sm_mhz, "sms": sms,
            "instructions_source": source}


class Clocks:
    """nvidia-smi samples during the timed region."""

    def __init__(self, index: int):
        self.proc = None
        self.path = None
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={index}",
                 "--query-gpu=clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"), stderr=subprocess.DEVNULL)
        except (OSError, FileNotFoundError):
            self.proc = None

    def stop(self):
        if not self.proc:
            return None
        time.sleep(0.25)
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        rows = []
        for line in Path(self.path).read_text().splitlines():
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                rows.append(parts)
        os.unlink(self.path)
        if not rows:
            return None
        sm = [float(r[0]) for r in rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[3 + i] == "Active"})
        return {"sm_mhz": statistics.median(sm) if sm else None,
                "sm_max_mhz": max(mx) if mx else None, "reasons": reasons,
                "samples": len(rows)}


def _cpu_baseline(lit, faces, threads, walk_tree=None, skip_empty=False, walls=None):
    """Oracle gather over faces [0, faces): shadow rays, seconds, walk stats.
    walk_tree / skip_empty / walls: walk as the device does (its tree, its
    options, its wall test) instead of the reference's way, for counting
    the device's node and triangle reads."""
    from oracle import pyoracle

    s = pyoracle.Scene(lit.xyz, lit.ids)
    if walk_tree is not None:
        s.set_tree(*walk_tree)
        s.set_skip_empty(skip_empty)
    if walls is not None:
        s.set_walls(*walls)
    lights = pyoracle.make_lights(lit.lights)
    t0 = time.perf_counter()
    _, rays, st = pyoracle.gather_luxels(s, lights, len(lit.lights), lit, 0, faces, ss=4,
                                         seed=SEED, threads=threads, stats=True)
    dt = time.perf_counter() - t0
    return rays, dt, st


def run_reference(args, rank):
    """CPU reference arm: the oracle restatement of the path, every thread."""
    if rank != 0:
        return
    from vrad_gb300 import scenes

    threads = os.cpu_count() or 1
    lit = scenes.lit_scene(SEED)
    from oracle import pyoracle

    s = pyoracle.Scene(lit.xyz, lit.ids)
    lights = pyoracle.make_lights(lit.lights)
    nf = lit.n_faces

    def step(i):
        f0 = (i * REF_FACES_PER_STEP) % nf
        t0 = time.perf_counter()
        _, rays = pyoracle.gather_luxels(s, lights, len(lit.lights), lit, f0,
                                         f0 + REF_FACES_PER_STEP, ss=4, seed=SEED, threads=threads)
        return rays, time.perf_counter() - t0

    for i in range(args.warmup):
        step(i)
    tot_r, tot_t = 0, 0.0
    for i in range(args.steps):
        r, t = step(args.warmup + i)
        tot_r += r
        tot_t += t
    v = tot_r / tot_t / 1e6
    sample = (f"{REF_FACES_PER_STEP} of {nf} faces per step (~{tot_r // max(args.steps, 1)} "
              f"shadow rays), 4 supersamples; the walk is the reference's SAH tree "
              f"(raytracer/environment.go:181-387) with no wall test")
    line = {
        "impl": "reference", "metric": "shadow Mrays/s (direct-light gather)", "value": round(v, 3),
        "unit": "Mrays/s", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": round(1e3 * tot_t / max(args.steps, 1), 3), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": "direct light, 4096 faces / 1.33M luxels x 4 samples, 64 point + "
                               "8 spot + 162-direction sky, 8208 triangles", "sample": sample},
        "cpu_baseline": {"value": round(v, 3), "unit": "Mrays/s", "cores": threads, "kind": "port",
                         "sample": sample},
        "e2e": {"value": round(v, 3), "unit": "Mrays/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def max_over_ranks(x: float, device) -> float:
    """The slowest rank's time: every rank ran the same replica workload."""
    import torch
    import torch.distributed as td

    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    td.all_reduce(t, op=td.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, max_ms: float) -> float:
    """Units processed by all replicas (M/s) over the slowest rank's time."""
    return units_per_rank * world / (max_ms * 1e-3) / 1e6


def _l2_read_gbs(device: int):
    """L2 read bandwidth: a 32 MiB buffer read 200 times in one launch
    (libvrgprobe.so, built beside the product library)."""
    from vrad_gb300 import build as vbuild

    probe = C.CDLL(str(vbuild.PROBE))
    probe.vrg_probe_l2_read_gbs.argtypes = [C.c_int, C.c_int64, C.c_int, C.c_void_p]
    gbs = C.c_double()
    rc = probe.vrg_probe_l2_read_gbs(device, 32 << 20, 200, C.byref(gbs))
    return gbs.value if rc == 0 else None


def _admit(lib_ctx, xyz, ids):
    """The scene's environment, and the time SetupAccelerationStructure takes
    with the walk tree built on the GPU and on the host (ms; the GPU build is
    timed after a first one that loads its kernels)."""
    import torch

    from vrad_gb300.environment import Environment

    times = {}
    for on_device in (1, 0, 1):
        e = Environment(lib_ctx)
        e.set_walk_tree_builder(on_device)
        e.add_triangles(xyz, ids)
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        e.SetupAccelerationStructure()
        times["device" if on_device else "host"] = round((time.perf_counter() - t0) * 1e3, 2)
        e.close()
    e = Environment(lib_ctx)  # the default builder for this size
    e.add_triangles(xyz, ids)
    e.SetupAccelerationStructure()
    return e, times


def _event_ms(stream, fn, steps, flush):
    """Per-step device times of fn (CUDA events on `stream`, L2 flushed
    before each step)."""
    import torch

    out = []
    for _ in range(steps):
        flush.zero_()
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(stream)
        fn()
        b.record(stream)
        torch.cuda.synchronize()
        out.append(a.elapsed_time(b))
    return out


def _trace_roofline(kernel, units, avg_ms, bytes_per_unit, hbm_peak, hbm_kind, l2, clk, sms,
                    prof, bytes_model, nodes, tris, variant=None):
    """Roofline record of a traversal kernel.  Its algorithmic bytes (kd
    nodes and leaf records) are served from L1 and L2, so the governing roof
    is instruction issue; the L2 and HBM fractions are given beside it, HBM
    from the DRAM bytes ncu counted for the same kernel.  The instruction
    count is the tuned variant's own (`warp_instructions_per_unit_v<n>`)
    where the summary has it."""
    alg = bytes_per_unit * units / (avg_ms * 1e-3) / 1e9
    traffic = _profile_value(prof, f"dram_bytes_per_launch_full_v{variant}") if variant is not None else None
    if traffic is None:
        traffic = _ncu_traffic(prof)
    sm_mhz = (clk or {}).get("sm_mhz")
    inst = _profile_value(prof, f"warp_instructions_per_unit_v{variant}") if variant is not None else None
    inst_of = f"variant {variant}" if inst is not None else "the variant the summary names"
    if inst is None:
        inst = _profile_value(prof, "warp_instructions_per_unit")
    issue = issue_roofline(inst, units, avg_ms, sm_mhz, sms, f"profiles/{prof}")
    if issue:
        issue["instructions_of"] = inst_of
    rec = {"bound": "issue", "kernel": kernel, "kernel_ms": round(avg_ms, 4),
           "bytes_per_unit": round(bytes_per_unit, 2), "bytes_model": bytes_model,
           "nodes_per_unit": round(float(nodes), 3), "tris_per_unit": round(float(tris), 3),
           "l2": {"achieved": round(alg, 1), "peak": round(l2, 1) if l2 else None, "unit": "GB/s",
                  "frac": round(alg / l2, 4) if l2 else None,
                  "peak_source": "L2-resident read kernel (probe.cu), timed in this run"},
           "hbm": {"achieved": round(traffic / (avg_ms * 1e-3) / 1e9, 1) if traffic else None,
                   "peak": hbm_peak, "unit": "GB/s",
                   "frac": round(traffic / (avg_ms * 1e-3) / 1e9 / hbm_peak, 5) if traffic else None,
                   "peak_kind": f"{hbm_kind} HBM copy", "traffic_source": f"profiles/{prof}"},
           "traffic": traffic}
    if issue:
        rec.update({"achieved": issue["achieved"], "peak": issue["peak"], "unit": issue["unit"],
                    "frac": issue["frac"], "issue": issue})
    else:
        rec.update({"achieved": rec["l2"]["achieved"], "peak": rec["l2"]["peak"], "unit": "GB/s",
                    "frac": rec["l2"]["frac"], "bound": "l2"})
    return rec


def run_gpu(args, rank, world, local_rank):
    import torch

    from vrad_gb300 import scenes
    from vrad_gb300.environment import Context, light_array

    dist = world > 1
    if dist:
        import torch.distributed as td

        td.init_process_group("nccl")
    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    # every launch (library kernels, L2 flush, events) goes to one stream
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    lib_ctx = Context(local_rank)
    lib_ctx.set_stream(stream.cuda_stream)
    if args.autotune_file:
        lib_ctx.autotune_load(args.autotune_file)
    lib = lib_ctx.lib
    sms = torch.cuda.get_device_properties(dev).multi_processor_count

    lit = scenes.lit_scene(SEED, n_faces=args.faces)
    env, admit_ms = _admit(lib_ctx, lit.xyz, lit.ids)
    env.set_faces(lit)
    lights = light_array(lit.lights)
    env.set_lights(lit.lights)
    nlux = env.num_luxels()
    d_out = torch.empty((nlux, 3), dtype=torch.float32, device=dev)
    rays = C.c_uint64()
    rc = lib.vrg_env_gather_direct_light_d(env.h, 4, SEED, d_out.data_ptr(), C.byref(rays))
    assert rc == 0, rc
    units = rays.value
    kernel = "direct_luxels"

    def step_dev():
        rc = lib.vrg_env_gather_direct_light_d(env.h, 4, SEED, d_out.data_ptr(), None)
        assert rc == 0, rc

    h_out = torch.empty((nlux, 3), dtype=torch.float32).pin_memory()
    nl = len(lit.lights)

    def step_host():
        rc = lib.vrg_env_set_lights(env.h, lights, nl)
        assert rc == 0, rc
        rc = lib.vrg_env_gather_direct_light(env.h, 4, SEED, h_out.data_ptr(), None)
        assert rc == 0, rc

    h2d, d2h = 80 * nl, 12 * nlux
    workload = ("direct light, %d faces / %d luxels x 4 supersamples, 64 point + 8 spot + "
                "162-direction sky, %d triangles" % (lit.n_faces, nlux, len(lit.ids)))

    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)  # > 129 MB L2
    for _ in range(max(args.warmup, 3)):
        step_dev()
        flush.zero_()
    torch.cuda.synchronize()

    lib_ctx.set_timing(True)
    lib_ctx.reset_stats()
    launches0 = lib_ctx.launch_count()
    clocks = Clocks(local_rank) if rank == 0 else None
    if dist:
        td.barrier()
    torch.cuda.synchronize()
    evs = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True))
           for _ in range(args.steps)]
    for k in range(args.steps):
        flush.zero_()
        evs[k][0].record(stream)
        step_dev()
        evs[k][1].record(stream)
    torch.cuda.synchronize()
    if dist:
        td.barrier()
    clk = clocks.stop() if clocks else None
    launches = lib_ctx.launch_count() - launches0
    step_ms = [a.elapsed_time(b) for a, b in evs]
    total_ms = sum(step_ms)
    kms, kn = lib_ctx.kernel_stats(kernel)
    lib_ctx.set_timing(False)
    if dist:
        total_ms = max_over_ranks(total_ms, dev)
    value = whole_job_rate(units * args.steps, world, total_ms)

    # end to end through the host-buffer C ABI (pinned host memory)
    for _ in range(2):
        step_host()
    e2e_t = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        step_host()
        e2e_t.append(time.perf_counter() - t0)
    # the median step: one host stall in a few wall-clock steps would move the
    # mean by itself (the mean is reported beside it)
    e2e_value = units * world / statistics.median(e2e_t) / 1e6
    e2e_mean = units * world / statistics.mean(e2e_t) / 1e6

    if rank != 0:
        if dist:
            td.destroy_process_group()
        return

    peak, peak_kind = _peaks()
    threads = os.cpu_count() or 1
    avg_ms = kms / max(kn, 1)
    tkey = Context.tune_key("direct_luxels", env.num_triangles(), nlux * 4)
    tv, tms = lib_ctx.autotune_choice(tkey)
    # the device's luxels of the timed bake, against the oracle's whole bake
    # (which is also the CPU baseline: every face, every host thread)
    got = h_out.numpy().copy()
    from oracle import pyoracle

    s_ref = pyoracle.Scene(lit.xyz, lit.ids)
    t0 = time.perf_counter()
    ref, rays_cpu = pyoracle.gather_luxels(s_ref, pyoracle.make_lights(lit.lights), nl, lit, 0,
                                           lit.n_faces, ss=4, seed=SEED, threads=threads)
    dt = time.perf_counter() - t0
    parity = {"oracle": "C restatement (oracle/vrad_oracle.c), every luxel of the bake",
              "tolerance_rel": 1e-4, "shadow_rays_equal": rays_cpu == units,
              **rel_error_stats(got, ref)}
    parity["within_tolerance"] = bool(parity["max_rel"] <= 1e-4 and parity["zero_ref_nonzero"] == 0
                                      and parity["shadow_rays_equal"])
    cpu = {"value": round(rays_cpu / dt / 1e6, 3), "unit": "Mrays/s", "cores": threads,
           "kind": "port",
           "sample": f"the whole bake, all {lit.n_faces} faces ({rays_cpu} shadow rays), walking "
                     "the reference's SAH tree with no wall test"}
    # walk statistics of the device's tree, options and wall test (for the byte model)
    skip_empty = tv in (6,)
    _, _, st = _cpu_baseline(lit, min(STATS_SAMPLE_FACES, lit.n_faces), threads,
                             env.walk_tree()[:3], skip_empty, env.wall_slots())
    nodes, tris = st[1] / st[0], st[2] / st[0]
    rays_per_sample = units / (4 * nlux)
    bytes_per_unit = 8 * nodes + 48 * tris + (24 + 12 / 4) / rays_per_sample
    torch.cuda.synchronize()
    l2 = _l2_read_gbs(local_rank)
    roof = _trace_roofline(
        kernel, units, avg_ms, bytes_per_unit, peak, peak_kind, l2, clk, sms,
        f"ncu_{kernel}.txt",
        "8 per kd node + 48 per triangle test (leaf-ordered records and wall slots), means of "
        "the oracle's walk of the device's tree, with the device's options and wall test, over "
        "the lines of faces 0-255, + sample position, normal and RGB share", nodes, tris, tv)
    line = {
        "metric": "shadow Mrays/s (direct-light gather)",
        "value": round(value, 3), "unit": "Mrays/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": round(total_ms / args.steps, 4),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (seeded SplitMix64 box rooms)",
        "config": {"workload": workload, "rays_per_step": units,
                   "luxel_samples_per_s_M": round(4 * nlux * args.steps * world / (total_ms * 1e-3) / 1e6, 3),
                   "l2": "flushed between steps (512 MiB write)", "parallelism": f"replicas{world}",
                   "autotune": {"bucket": tkey, "variant": tv,
                                "variant_ms": [round(x, 4) for x in tms]},
                   "setup_acceleration_structure_ms": admit_ms},
        "parity": parity,
        "e2e": {"value": round(e2e_value, 3), "unit": "Mrays/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h, "statistic": f"median of {len(e2e_t)} wall-clock steps",
                "mean_value": round(e2e_mean, 3)},
        "gpu_launches": int(launches),
        "roofline": roof,
        "cpu_baseline": cpu,
        "clocks": clk,
    }
    env.close()
    if not args.headline_only and world == 1:
        for name, fn in (("anyhit", sub_anyhit), ("rooms", sub_rooms), ("radiosity", sub_radiosity),
                         ("batch", sub_batch), ("serve", sub_serve)):
            t0 = time.perf_counter()
            try:
                line[name] = fn(args, lib_ctx, stream, dev, flush, l2, sms)
            except Exception as exc:  # a failed sub-workload is reported, not hidden
                line[name] = {"error": f"{type(exc).__name__}: {exc}"}
            line[name]["wall_s"] = round(time.perf_counter() - t0, 1)
    print(json.dumps(line), flush=True)
    if dist:
        td.destroy_process_group()


def sub_anyhit(args, lib_ctx, stream, dev, flush, l2, sms):
    """Config 0: 2^20 shadow lines in the 12,300-triangle room, occlusion
    mask (and closest hit) per line; every bit and hit checked against the
    oracle."""
    import torch

    from vrad_gb300 import scenes
    from vrad_gb300.environment import Context

    lib = lib_ctx.lib
    sc = scenes.anyhit_scene(SEED)
    env, admit_ms = _admit(lib_ctx, sc.xyz, sc.ids)
    n = sc.starts.shape[0]
    d_a = torch.from_numpy(sc.starts).to(dev)
    d_b = torch.from_numpy(sc.stops).to(dev)
    d_m = torch.empty((n + 31) // 32, dtype=torch.int32, device=dev)
    d_h = torch.empty(n, dtype=torch.int32, device=dev)
    d_t = torch.empty(n, dtype=torch.float32, device=dev)

    def mask():
        rc = lib.vrg_env_occlusion_mask_d(env.h, d_a.data_ptr(), d_b.data_ptr(), n, -1,
                                          d_m.data_ptr(), None, None)
        assert rc == 0, rc

    def closest():
        rc = lib.vrg_env_occlusion_mask_d(env.h, d_a.data_ptr(), d_b.data_ptr(), n, -1,
                                          d_m.data_ptr(), d_h.data_ptr(), d_t.data_ptr())
        assert rc == 0, rc

    for fn in (mask, closest):
        for _ in range(max(args.warmup, 3)):
            fn()
            flush.zero_()
    torch.cuda.synchronize()
    clocks = Clocks(dev.index)
    lib_ctx.set_timing(True)
    lib_ctx.reset_stats()
    mask_ms = _event_ms(stream, mask, args.steps, flush)
    kms, kn = lib_ctx.kernel_stats("trace_mask")
    lib_ctx.set_timing(False)
    clk = clocks.stop()
    hit_ms = _event_ms(stream, closest, args.steps, flush)
    got_m = d_m.cpu().numpy().view(np.uint32)
    got_h, got_t = d_h.cpu().numpy(), d_t.cpu().numpy()
    # end to end through the host-buffer ABI (page-locked end points)
    h_a = torch.from_numpy(sc.starts).pin_memory()
    h_b = torch.from_numpy(sc.stops).pin_memory()
    h_m = torch.empty((n + 31) // 32, dtype=torch.int32).pin_memory()

    def host():
        rc = lib.vrg_env_occlusion_mask(env.h, h_a.data_ptr(), h_b.data_ptr(), n, -1,
                                        h_m.data_ptr(), None, None)
        assert rc == 0, rc

    host()
    e2e = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        host()
        e2e.append(time.perf_counter() - t0)
    from oracle import pyoracle

    threads = os.cpu_count() or 1
    s = pyoracle.Scene(sc.xyz, sc.ids)
    t0 = time.perf_counter()
    rm = s.occlusion_mask(sc.starts, sc.stops, threads=threads)
    dt = time.perf_counter() - t0
    _, rh, rt = s.occlusion_mask(sc.starts, sc.stops, threads=threads, closest=True)
    diff_bits = int(np.unpackbits((got_m ^ rm).view(np.uint8)).sum())
    tv, tms = lib_ctx.autotune_choice(Context.tune_key("trace_mask", env.num_triangles(), n))
    hv, hms = lib_ctx.autotune_choice(Context.tune_key("trace_mask_hit", env.num_triangles(), n))
    # the device's walk, counted by the oracle on the device's tree
    skip_empty = tv in (12, 13, 14, 15, 16, 17, 18, 19)
    s.set_tree(*env.walk_tree()[:3])
    s.set_skip_empty(skip_empty)
    _, st = s.occlusion_mask(sc.starts, sc.stops, threads=threads, stats=True)
    nodes, tris = st[:, 0].mean(), st[:, 1].mean()
    bytes_per_unit = 24 + 1 / 8 + 8 * nodes + 48 * tris
    prof = "ncu_trace_unit_skip.txt" if tv in (13, 14, 15, 16, 17, 18, 19) else (
        "ncu_trace_unit_stream.txt" if tv in (6, 7, 9, 10, 11) else "ncu_trace_mask.txt")
    peak, kind = _peaks()
    avg_ms = kms / max(kn, 1)
    env.close()
    return {
        "metric": "shadow Mrays/s (any-hit occlusion mask)",
        "value": round(n / (statistics.mean(mask_ms) * 1e-3) / 1e6, 3), "unit": "Mrays/s",
        "ms_per_step": round(statistics.mean(mask_ms), 4),
        "config": {"workload": "2^20 shadow lines, both ends uniform in the 4,096-unit room, "
                               "12,300-triangle box room (1,024 boxes), seed 0",
                   "l2": "flushed between steps (512 MiB write)",
                   "autotune": {"variant": tv, "variant_ms": [round(x, 4) for x in tms]},
                   "setup_acceleration_structure_ms": admit_ms},
        "closest_hit": {"value": round(n / (statistics.mean(hit_ms) * 1e-3) / 1e6, 3),
                        "unit": "Mrays/s", "ms_per_step": round(statistics.mean(hit_ms), 4),
                        "outputs": "mask + hit index + t", "autotune_variant": hv},
        "e2e": {"value": round(n / statistics.median(e2e) / 1e6, 3), "unit": "Mrays/s",
                "h2d_bytes_per_step": 24 * n, "d2h_bytes_per_step": 4 * ((n + 31) // 32),
                "statistic": f"median of {len(e2e)} wall-clock steps",
                "mean_value": round(n / statistics.mean(e2e) / 1e6, 3)},
        "parity": {"oracle": "C restatement, all 2^20 lines", "mask_bits_differing": diff_bits,
                   "hit_index_differing": int(np.count_nonzero(got_h != rh)),
                   "t_bits_differing": int(np.count_nonzero(got_t.view(np.uint32) != rt.view(np.uint32))),
                   "exact": diff_bits == 0 and bool(np.array_equal(got_h, rh))
                   and bool(np.array_equal(got_t.view(np.uint32), rt.view(np.uint32)))},
        "roofline": _trace_roofline(
            "trace_mask", n, avg_ms, bytes_per_unit, peak, kind, l2, clk, sms, prof,
            "24 end points + 1/8 mask + 8 per kd node + 48 per triangle test, means of the "
            "oracle's walk of the device's tree with the device's options", nodes, tris, tv),
        "cpu_baseline": {"value": round(n / dt / 1e6, 3), "unit": "Mrays/s", "cores": threads,
                         "kind": "port", "sample": f"all {n} lines, the reference's SAH tree"},
        "clocks": clk,
    }


def sub_rooms(args, lib_ctx, stream, dev, flush, l2, sms):
    """What the wall cells buy.  The headline's box room has six walls of two
    triangles each, so most sky lines end on one wall test.  Here the same
    bake runs with the wall cells off; on the same scene with each room face
    split into 16 x 16 tiles (512 triangles per face, one tile per cell);
    and on the same boxes, faces and lights written as a compiled map's
    brushes (16-unit thick walls, a sky face over the room) and ingested
    through add_bsp_world (addBrushesForRayTrace) -- each with and without
    the cells.  The tiled room's and the brush world's luxels of faces 0-255
    are checked against the oracle."""
    import torch

    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment

    from vrad_gb300.environment import Context

    out = {}
    checked = {}
    for name, tiles, slots in (("box_room_walls_off", 1, False), ("tiled_16x16_walls_on", 16, True),
                               ("tiled_16x16_walls_off", 16, False), ("brush_world_walls_on", 0, True),
                               ("brush_world_walls_off", 0, False)):
        # a context of its own per room, so that each is autotuned on itself
        ctx = Context(dev.index)
        ctx.set_stream(stream.cuda_stream)
        lib = ctx.lib
        env = Environment(ctx)
        env.set_wall_slots(slots)
        if tiles == 0:
            lumps, lit = scenes.lit_brush_world(SEED)
            env.add_bsp_world(lumps)
        else:
            lit = scenes.lit_scene(SEED, wall_tiles=tiles)
            env.add_triangles(lit.xyz, lit.ids)
        env.SetupAccelerationStructure()
        env.set_faces(lit)
        env.set_lights(lit.lights)
        nlux = env.num_luxels()
        d_out = torch.empty((nlux, 3), dtype=torch.float32, device=dev)
        rays = C.c_uint64()

        def bake(want_rays=False):
            rc = lib.vrg_env_gather_direct_light_d(env.h, 4, SEED, d_out.data_ptr(),
                                                   C.byref(rays) if want_rays else None)
            assert rc == 0, rc

        bake(True)
        for _ in range(2):
            bake()
        ms = _event_ms(stream, bake, max(3, args.steps // 2), flush)
        mean = statistics.mean(ms)
        tv, tms = ctx.autotune_choice(Context.tune_key("direct_luxels", env.num_triangles(), nlux * 4))
        out[name] = {"value": round(rays.value / (mean * 1e-3) / 1e6, 1), "unit": "Mrays/s",
                     "ms_per_step": round(mean, 3), "rays_per_step": rays.value,
                     "triangles": env.num_triangles(),
                     "wall_triangles_per_face_reported": env.wall_slots()[1].tolist(),
                     "autotune": {"variant": tv, "variant_ms": [round(x, 3) for x in tms]}}
        if slots and name != "box_room_walls_off":
            checked[name.replace("_walls_on", "")] = (d_out.cpu().numpy(), lit, *env.get_triangle_vertices())
        env.close()
        ctx.close()
    from oracle import pyoracle

    for key, (got, lit, xyz, ids) in checked.items():
        off = lit.luxel_offset()
        nf = min(256, lit.n_faces)
        ref, _ = pyoracle.gather_luxels(pyoracle.Scene(xyz, ids), pyoracle.make_lights(lit.lights),
                                        len(lit.lights), lit, 0, nf, ss=4, seed=SEED,
                                        threads=os.cpu_count() or 1)
        out[f"{key}_parity_faces_0_255"] = rel_error_stats(got[: off[nf]], ref)
    return out


def sub_radiosity(args, lib_ctx, stream, dev, flush, l2, sms):
    """Config 2: the direct-light faces subdivided at 64 units; transfers from
    K closest-hit rays per patch (CSR), then the bounce loop to a 1e-3
    relative delta.  Sampled rows are rebuilt by the oracle bit for bit and
    the bounce is checked against the float64 oracle over the device's CSR."""
    import torch

    from vrad_gb300 import scenes
    from vrad_gb300.environment import Context, Environment

    ctx = lib_ctx
    lit = scenes.lit_scene(SEED, n_faces=args.faces)
    env = Environment(ctx)
    env.add_triangles(lit.xyz, lit.ids)
    env.SetupAccelerationStructure()
    env.set_faces(lit)
    env.set_lights(lit.lights)
    t0 = time.perf_counter()
    P = env.make_patches()
    t_patch = time.perf_counter() - t0
    nl = P["n_leaves"]
    dirs = scenes.transfer_directions(args.k)
    t0 = time.perf_counter()
    env.make_transfers(dirs)  # the first build of a size bucket runs the autotuner
    t_first = time.perf_counter() - t0
    ctx.set_timing(True)
    ctx.reset_stats()
    t0 = time.perf_counter()
    nnz = env.make_transfers(dirs)
    t_xfer = time.perf_counter() - t0
    _, _, ovf = env.transfer_info()
    rows_main_ms = ctx.kernel_stats("transfer_rows")[0]
    rows_ms = rows_main_ms + ctx.kernel_stats("transfer_rows_sorted")[0]
    xkey = Context.tune_key("transfer_rows", env.num_triangles(), nl * args.k)
    xv = ctx.autotune_choice(xkey)[0]
    gather_ms = ctx.kernel_stats("transfer_gather")[0]
    ctx.set_timing(False)
    direct = env.gather_patch_direct(nl)
    env.bounce_light(nl, 100, 1e-3)  # the first solve of a size bucket tunes the SpMV
    tkey = Context.tune_key("bounce_spmv", nnz, nl)
    tv, tms = ctx.autotune_choice(tkey)
    # per-kernel timing pass (one launch per bounce)
    ctx.set_timing(True)
    ctx.reset_stats()
    clocks = Clocks(dev.index)
    total, bounces, delta = env.bounce_light(nl, 100, 1e-3)
    clk = clocks.stop()
    spmv_ms, spmv_n = ctx.kernel_stats("bounce_spmv")
    red_ms, _ = ctx.kernel_stats("bounce_reduce")
    ctx.set_timing(False)
    # graph pass, wall clock of the whole loop
    for _ in range(2):
        env.bounce_light(nl, 100, 1e-3)
    reps = max(args.steps, 1)
    t0 = time.perf_counter()
    for _ in range(reps):
        env.bounce_light(nl, 100, 1e-3)
    loop_s = (time.perf_counter() - t0) / reps
    # parity: sampled rows, leaf direct light, bounce vs float64
    from oracle import pyoracle

    threads = os.cpu_count() or 1
    row_ptr, col, w = env.get_transfers(nl, nnz)
    s = pyoracle.Scene(lit.xyz, lit.ids)
    OP = pyoracle.make_patches(lit)
    rng = np.random.default_rng(SEED + 2)
    per_row = np.diff(row_ptr)
    rows = set(rng.choice(nl, min(args.check_rows, nl), replace=False).tolist())
    rows |= set(np.nonzero(per_row > 7168)[0][:64].tolist())
    rows = np.array(sorted(rows), np.int64)
    orow, ocol, ocnt = pyoracle.make_transfer_rows(s, lit, OP, dirs, rows, threads=threads)
    kf = np.float32(args.k)
    mism = 0
    for j, r in enumerate(rows):
        a, b = row_ptr[r], row_ptr[r + 1]
        oa, ob = orow[j], orow[j + 1]
        mism += not (b - a == ob - oa and np.array_equal(col[a:b], ocol[oa:ob]) and np.array_equal(
            w[a:b].view(np.uint32), (ocnt[oa:ob] / kf).astype(np.float32).view(np.uint32)))
    leaf_patch = np.nonzero(OP["leaf_index"] >= 0)[0]
    face = OP["face"][leaf_patch]
    pts = (OP["center"][leaf_patch] + lit.normal[face] * np.float32(0.125)).astype(np.float32)
    ref_direct, _ = pyoracle.gather_points(s, pyoracle.make_lights(lit.lights), len(lit.lights),
                                           pts, lit.normal[face], threads=threads)
    refl = lit.refl[face]
    rtot, rb, rdeltas = pyoracle.bounce_f64(row_ptr, col, w, refl, ref_direct,
                                            np.zeros_like(refl), 100, 1e-3, threads=threads)
    nzm = rtot != 0
    brel = np.abs(total.astype(np.float64)[nzm] - rtot[nzm]) / np.abs(rtot[nzm])
    dstat = rel_error_stats(direct, ref_direct)
    peak, kind = _peaks()
    per_iter_ms = spmv_ms / max(spmv_n, 1)
    bytes_iter = 8 * nnz + 72 * nl  # col+weight per entry; row_ptr, refl, total RMW, emit out per row
    achieved = bytes_iter / (per_iter_ms * 1e-3) / 1e9
    traffic_k = _profile_value("ncu_bounce_spmv.txt", "dram_bytes_per_entry")
    l2_k = _profile_value("ncu_bounce_spmv.txt", "l2_bytes_per_entry")
    # the lightmap samples of a whole bake of this scene (direct + bounce):
    # the kernel timed per launch with L2 flushed before each call, every
    # sample compared with the oracle's encoding of the same bake
    import torch

    env.bake(4, SEED, 100, 1e-3)
    res = env.get_bake(nl)
    env.get_lightmap()
    ctx.set_timing(True)
    ctx.reset_stats()
    lm_calls = []
    for _ in range(10):
        flush.zero_()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        samples, _ = env.get_lightmap()
        lm_calls.append(time.perf_counter() - t0)
    lm_ms, lm_n = ctx.kernel_stats("lightmap")
    ctx.set_timing(False)
    want = pyoracle.lightmap(lit, OP, res["luxels"], res["patch_total"])
    lm_diff = int(np.count_nonzero(samples.view("<u4").ravel() != want))
    nlux = env.num_luxels()
    lm_bytes = 16 * nlux + 16 * nl  # direct light in and sample out per luxel, bounced light per leaf
    lm_kernel_ms = lm_ms / max(lm_n, 1)
    env.close()
    return {
        "metric": "bounce loop (Jacobi gather to 1e-3 over the built transfer CSR; its build "
                  "time is transfers.build_s)",
        "value": round(1.0 / loop_s, 3), "unit": "solves/s", "ms_per_step": round(loop_s * 1e3, 3),
        "config": {"workload": f"{lit.n_faces} faces subdivided at 64 units", "leaf_patches": nl,
                   "transfer_rays_per_patch": args.k, "nnz": nnz, "nnz_per_row": round(nnz / nl, 1),
                   "rows_past_row_table": ovf, "bounces": bounces, "final_delta": delta,
                   "autotune": {"bucket": tkey, "variant": tv,
                                "variant_ms": [round(x, 4) for x in tms]}},
        "transfers": {"build_s": round(t_xfer, 3), "first_build_s_with_autotune": round(t_first, 3),
                      "rows_kernel_ms": round(rows_ms, 3), "gather_kernel_ms": round(gather_ms, 3),
                      "rays_per_s_M": round(nl * args.k / (rows_ms * 1e-3) / 1e6, 1),
                      "autotune": dict(zip(("bucket", "variant", "variant_ms"),
                                           (xkey,) + ctx.autotune_choice(xkey))),
                      "patch_build_s": round(t_patch, 3),
                      # the row kernel's closest-hit walks (every row's k rays)
                      # against the SMs' issue rate
                      "roofline": dict(issue_roofline(
                          _profile_value("ncu_transfer_rows.txt",
                                         f"warp_instructions_per_unit_k{args.k}_v{xv}"),
                          nl * args.k, rows_main_ms, (clk or {}).get("sm_mhz"), sms,
                          "profiles/ncu_transfer_rows.txt") or {}, bound="issue",
                          kernel="transfer_rows", kernel_ms=round(rows_main_ms, 3))},
        "parity": {"transfer_rows_checked": int(len(rows)), "transfer_rows_differing": int(mism),
                   "leaf_direct": dstat,
                   "bounce": {"oracle": "float64 Jacobi over the device's CSR, oracle direct light",
                              "tolerance_rel": 1e-3, "bounces": bounces, "oracle_bounces": int(rb),
                              "max_rel": float(brel.max()) if brel.size else 0.0,
                              "p99_rel": float(np.percentile(brel, 99)) if brel.size else 0.0,
                              "zero_ref_nonzero": int(np.count_nonzero(total[~nzm]))}},
        "roofline": {"bound": "hbm", "achieved": round(achieved, 1), "peak": peak, "unit": "GB/s",
                     "frac": round(achieved / peak, 4),
                     "traffic": round(traffic_k * nnz) if traffic_k else None,
                     "traffic_source": "profiles/ncu_bounce_spmv.txt (DRAM bytes per CSR entry, "
                                       "scaled to this nnz)",
                     "peak_kind": f"{kind} HBM copy", "kernel": "bounce_spmv",
                     "kernel_ms": round(per_iter_ms, 4), "bytes_per_launch": bytes_iter,
                     "reduce_ms": round(red_ms / max(spmv_n, 1), 4),
                     # what holds it: the L2-to-SM traffic of the gathers and
                     # the stream (ncu sectors per entry) against the probe
                     "l2": ({"achieved": round(l2_k * nnz / (per_iter_ms * 1e-3) / 1e9, 1),
                             "peak": round(l2, 1), "unit": "GB/s",
                             "frac": round(l2_k * nnz / (per_iter_ms * 1e-3) / 1e9 / l2, 4),
                             "bytes_per_entry": l2_k,
                             "source": "profiles/ncu_bounce_spmv.txt (L2 sectors read per CSR entry); "
                                       "peak: L2-resident read kernel (probe.cu), timed in this run"}
                            if l2_k and l2 else None)},
        "lightmap": {"samples": nlux, "kernel_us": round(lm_kernel_ms * 1e3, 2),
                     "bytes_per_launch": lm_bytes,
                     "achieved_gbs": round(lm_bytes / (lm_kernel_ms * 1e-3) / 1e9, 1),
                     "frac_of_hbm": round(lm_bytes / (lm_kernel_ms * 1e-3) / 1e9 / peak, 4),
                     "call_ms_with_copy": round(1e3 * statistics.median(lm_calls), 3),
                     "l2": "flushed before each call",
                     "parity": {"oracle": "orc_lightmap over the device's bake",
                                "samples_differing": lm_diff, "exact": lm_diff == 0}},
        "clocks": clk,
    }


def sub_batch(args, lib_ctx, stream, dev, flush, l2, sms):
    """Config 3: 256 scenes with log-uniform face counts (64-4,096), each
    baked direct + bounce to a 1e-3 delta: the batched path (one persistent
    direct launch + one block-diagonal bounce graph) against the plain
    one-scene-per-launch loop on the same resident scenes, and the two
    paths' results compared scene by scene."""
    import torch

    from vrad_gb300 import scenes
    from vrad_gb300.environment import Batch, Context, Environment

    ctx = lib_ctx
    t0 = time.perf_counter()
    lits = scenes.batch_scenes(SEED, n_scenes=args.scenes)
    dirs = scenes.transfer_directions(args.batch_k)
    envs, leaves, nnzs = [], [], []
    for lit in lits:
        env = Environment(ctx)
        env.add_triangles(lit.xyz, lit.ids)
        env.SetupAccelerationStructure()
        env.set_faces(lit)
        env.set_lights(lit.lights)
        leaves.append(env.make_patches()["n_leaves"])
        nnzs.append(env.make_transfers(dirs))
        envs.append(env)
    setup_s = time.perf_counter() - t0
    batch = Batch(ctx)
    for env in envs:
        batch.add(env)

    def plain():
        r = 0
        for env in envs:
            r += env.bake(4, SEED, 100, 1e-3)
        return r

    def batched():
        return batch.bake(4, SEED, 100, 1e-3)

    res, outs = {}, {}
    for name, fn in (("plain", plain), ("batched", batched)):
        for _ in range(max(args.warmup, 1)):
            fn()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        rays = 0
        for _ in range(args.batch_steps):
            rays = fn()
        dt = (time.perf_counter() - t0) / args.batch_steps
        res[name] = (dt, rays)
        outs[name] = [env.get_bake(nl) for env, nl in zip(envs, leaves)]
    lux_bits = sum(int(np.count_nonzero(a["luxels"].view(np.uint32) != b["luxels"].view(np.uint32)))
                   for a, b in zip(outs["plain"], outs["batched"]))
    tot_rel = max(float(np.max(np.abs(a["patch_total"].astype(np.float64) - b["patch_total"]) /
                               np.maximum(np.abs(a["patch_total"]), 1e-30)))
                  if a["patch_total"].size else 0.0
                  for a, b in zip(outs["plain"], outs["batched"]))
    n = len(envs)
    gkey = Context.tune_key("batch_gather", sum(env.num_triangles() for env in envs),
                            sum(env.num_luxels() * 4 + nl for env, nl in zip(envs, leaves)))
    gv, gms = ctx.autotune_choice(gkey)
    for env in envs:
        env.close()
    batch.close()
    return {
        "metric": "bakes/s (batched vs one scene per launch)",
        "value": round(n / res["batched"][0], 2), "unit": "bakes/s",
        "ms_per_step": round(1e3 * res["batched"][0], 2), "steps": args.batch_steps,
        "config": {"workload": f"{n} scenes, faces log-uniform 64-4096, 4 samples per luxel, "
                               f"64-unit patches, bounce to 1e-3",
                   "luxel_spacing": 48.0,
                   "deviation": "48-unit luxels (the direct-light config uses 16) and 8,192 "
                                "transfer rays per patch, to keep setup within the bench's minutes",
                   "transfer_rays_per_patch": args.batch_k,
                   "nnz_per_row": round(sum(nnzs) / max(sum(leaves), 1), 1),
                   "luxels": sum(l.n_luxels for l in lits), "faces": sum(l.n_faces for l in lits),
                   "leaf_patches": sum(leaves), "setup_s": round(setup_s, 1),
                   "autotune": {"bucket": gkey, "variant": gv, "variant_ms": [round(x, 3) for x in gms]}},
        "plain": {"bakes_per_s": round(n / res["plain"][0], 2), "ms_per_batch": round(1e3 * res["plain"][0], 2)},
        "batched": {"bakes_per_s": round(n / res["batched"][0], 2),
                    "ms_per_batch": round(1e3 * res["batched"][0], 2)},
        "speedup": round(res["plain"][0] / res["batched"][0], 3),
        "shadow_rays_per_batch": res["batched"][1],
        "parity": {"against": "the plain path's bake of each scene (itself checked against the "
                              "oracle in tests/test_gpu_batch.py)",
                   "luxel_values_differing": lux_bits, "bounced_light_max_rel": tot_rel},
    }


def sub_serve(args, lib_ctx, stream, dev, flush, l2, sms):
    """Config 4: 8 resident scenes (faces log-uniform 300-4,096, 16-unit
    luxels, 10k-140k leaf patches); Poisson request streams at several
    rates; each request moves and rescales 1-16 point/spot lights,
    re-gathers the affected luxels and re-solves the bounce to a 1e-3
    relative change.  The served path (8 slots, continuous admission) runs
    beside the plain serial path (1 slot) on the same request stream."""
    from vrad_gb300 import scenes
    from vrad_gb300.environment import Environment, Server, edit_array, make_light

    ctx = lib_ctx
    counts = scenes.batch_face_counts(SEED + 7, 8, 300, 4096)
    lits, envs, leaves = [], [], []
    t0 = time.perf_counter()
    dirs = scenes.transfer_directions(args.batch_k)
    for i, c in enumerate(counts):
        lit = scenes.lit_scene(5000 + i, n_faces=int(c))
        env = Environment(ctx)
        env.add_triangles(lit.xyz, lit.ids)
        env.SetupAccelerationStructure()
        env.set_faces(lit)
        env.set_lights(lit.lights)
        P = env.make_patches()
        env.make_transfers(dirs)
        env.relight_prepare(4, SEED, 100, 1e-3)
        lits.append(lit)
        envs.append(env)
        leaves.append(P["n_leaves"])
    setup_s = time.perf_counter() - t0
    rng = np.random.default_rng(SEED)
    rates = [float(r) for r in args.rates.split(",")]
    n_req = args.requests

    def make_requests():
        reqs = []
        for _ in range(n_req):
            s = int(rng.integers(0, len(envs)))
            lit = lits[s]
            k = int(rng.integers(1, 17))
            idx = rng.choice(len(lit.lights) - 1, size=k, replace=False)
            edits = []
            for i in idx:
                li = lit.lights[int(i)]
                o = tuple(float(c) for c in rng.uniform(1.0, 4095.0, 3))
                it = tuple(float(c) * float(rng.uniform(0.5, 2.0)) for c in li.intensity)
                edits.append((int(i), make_light(li.type, o, it, li.normal, **li.keys)))
            reqs.append((s, edit_array(edits), len(edits)))
        return reqs

    def run(slots, arrivals, reqs):
        srv = Server(ctx, slots=slots, max_iters=32, rel_tol=1e-3)
        ids = [srv.add_scene(env) for env in envs]
        tickets = []
        t_start = time.perf_counter()
        for (s, arr, n), ta in zip(reqs, arrivals):
            while time.perf_counter() - t_start < ta:
                pass
            t = C.c_int64()
            rc = srv.lib.vrg_server_submit(srv.h, ids[s], arr, n, C.byref(t))
            assert rc == 0, rc
            tickets.append(t.value)
        srv.drain()
        res = [srv.result(t) for t in tickets]
        srv.close()
        lat = np.array([r["done"] - r["submit"] for r in res]) * 1e3
        span = max(r["done"] for r in res) - min(r["submit"] for r in res)
        bounces = np.array([r["bounces"] for r in res])
        assert all(r["status"] == 0 for r in res)
        return {"p50_ms": round(float(np.percentile(lat, 50)), 3),
                "p99_ms": round(float(np.percentile(lat, 99)), 3),
                "mean_ms": round(float(lat.mean()), 3),
                "bakes_per_s": round(len(res) / span, 1), "mean_bounces": round(float(bounces.mean()), 2)}

    warm = make_requests()[:32]
    warm_arr = np.cumsum(rng.exponential(1.0 / 1000.0, len(warm)))
    run(8, warm_arr, warm)
    run(1, warm_arr, warm)
    table = {}
    for rate in rates:
        # one request stream per rate, the same requests at the same times on both paths
        reqs = make_requests()
        arrivals = np.cumsum(rng.exponential(1.0 / rate, len(reqs)))
        table[str(int(rate))] = {"served": run(8, arrivals, reqs), "serial": run(1, arrivals, reqs)}
    top = table[str(int(rates[-1]))]
    for env in envs:
        env.close()
    return {
        "metric": "relight p50/p99 ms and bakes/s (served vs plain serial)",
        "value": top["served"]["p99_ms"], "unit": "ms (p99 at the highest rate)",
        "higher_is_better": False,
        "config": {"workload": "8 resident scenes, faces " + ",".join(str(int(c)) for c in counts) +
                   f", leaf patches {min(leaves)}-{max(leaves)}, {args.batch_k} transfer rays/patch, "
                   "1-16 light edits per request, bounce re-solve to 1e-3",
                   "requests_per_rate": n_req, "setup_s": round(setup_s, 1)},
        "rates": table,
        "parity": {"against": "a full re-bake with the edited light table, bit for bit, and the "
                              "same result alone and in the mix (tests/test_gpu_relight.py)"},
    }


def run_one(args, local_rank):
    """`--workload X`: one of the sub-workloads as its own line."""
    import torch

    from vrad_gb300.environment import Context

    torch.cuda.set_device(local_rank)
    dev = torch.device("cuda", local_rank)
    stream = torch.cuda.Stream(device=dev)
    torch.cuda.set_stream(stream)
    ctx = Context(local_rank)
    ctx.set_stream(stream.cuda_stream)
    if args.autotune_file:
        ctx.autotune_load(args.autotune_file)
    sms = torch.cuda.get_device_properties(dev).multi_processor_count
    flush = torch.empty(512 << 20, dtype=torch.uint8, device=dev)
    l2 = _l2_read_gbs(local_rank)
    fn = {"anyhit": sub_anyhit, "rooms": sub_rooms, "radiosity": sub_radiosity, "batch": sub_batch,
          "serve": sub_serve}[args.workload]
    rec = fn(args, ctx, stream, dev, flush, l2, sms)
    rec.setdefault("higher_is_better", True)
    rec.update({"n_gpus": 1, "steps": args.steps, "warmup": args.warmup, "scaling": "weak",
                "vs_baseline": None, "dtype": "f32", "data": "synthetic (seeded SplitMix64 box rooms)"})
    print(json.dumps(rec), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    ap.add_argument("--workload", default="direct",
                    choices=["direct", "anyhit", "rooms", "radiosity", "batch", "serve"])
    ap.add_argument("--headline-only", action="store_true",
                    help="the direct-light line alone, without the other workloads")
    ap.add_argument("--rates", default="50,200,1000,2000", help="request rates of the serve workload")
    ap.add_argument("--requests", type=int, default=200, help="requests per rate (serve)")
    ap.add_argument("--scenes", type=int, default=256, help="scenes of the batch workload")
    ap.add_argument("--batch-steps", type=int, default=3, help="timed batches (batch)")
    ap.add_argument("--faces", type=int, default=4096,
                    help="lit faces of the direct-light scene (smaller only for profiling)")
    ap.add_argument("--autotune-file", default=None,
                    help="load saved autotune choices ('bucket variant' lines) before running")
    ap.add_argument("--k", type=int, default=65536,
                    help="transfer rays per patch of the radiosity workload")
    ap.add_argument("--batch-k", type=int, default=8192,
                    help="transfer rays per patch of the batch and serve workloads")
    ap.add_argument("--check-rows", type=int, default=256,
                    help="transfer rows the oracle rebuilds to check the radiosity CSR")
    args = ap.parse_args()
    rank = _env_int("RANK", 0)
    world = _env_int("WORLD_SIZE", 1)
    local_rank = _env_int("LOCAL_RANK", 0)
    if args.impl == "reference":
        run_reference(args, rank)
    elif args.workload == "direct":
        run_gpu(args, rank, world, local_rank)
    elif rank == 0:
        run_one(args, local_rank)


if __name__ == "__main__":
    main()
