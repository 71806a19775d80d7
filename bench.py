"""Benchmark of the GB300 volumetric path tracer (plain path, 1024^2 sparse 512^3 workload).

One step = one launch of the plain tracer over the whole 1024x1024 image at STEP_SPP samples
per pixel on the sparse 512^3 fBm cloud (sigma_t max 200, albedo 0.999, HG g = 0.85, <= 256
bounces, sun at 20 degrees + Hosek-Wilkie sky). Metric: paths/s = pixels * spp / time.
The line also carries `nrc_vs_plain`: GPU time for the radiance-cache renderer and for the plain
tracer to reach relMSE 1e-3 against a 16384-spp FP64 image on the 256x256 dense 64^3 scene.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference] [--config c2|c1|c4|c5]
                  [--no-nrc] [--no-cpu-baseline] [--nrc-frames N] [--mlp] [--tracker megakernel|wavefront]

`--config c4` times the 16-scene batch (one CUDA graph per step), `--config c5` the 2048^2 /
1024^3 stress scene; `--nrc-frames N` runs only the radiance-cache frame loop and `--mlp` only
the cache's MLP kernels (profiling); `--tracker wavefront` times the wavefront form of the plain
tracker instead of the persistent megakernel.

`--impl reference` times the reference's per-path CPU algorithm on the host cores. The reference's
own implementation (OptiX raygen + tiny-cuda-nn) cannot be built on this platform, so the arm runs
the project's CPU restatement of it (the oracle), with all host threads, on whole 16-spp frames of
the same workload. Its inputs (the fBm volume and the Hosek-Wilkie sky texture) are built on the
host by the oracle as well: that arm loads no product library and touches no GPU.
"""
from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

STEP_SPP = 16
L2_FLUSH_BYTES = 512 << 20   # larger than the 129 MB L2


def _peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def _profile_traffic(kernel_key: str, workload: str):
    """DRAM bytes per launch recorded from an ncu capture in profiles/*.md
    (a line `traffic_bytes_per_launch[<kernel>/<workload>]: <bytes>`)."""
    pat = re.compile(r"traffic_bytes_per_launch\[" + re.escape(kernel_key) + "/" + re.escape(workload) +
                     r"\]:\s*([0-9.eE+]+)")
    for f in sorted((ROOT / "profiles").glob("*.md")):
        m = pat.search(f.read_text())
        if m:
            return float(m.group(1)), f.name
    return None, None


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi while the timed region runs."""

    def __init__(self, uuid: str | None):
        self.uuid = uuid
        self.samples = []
        self._stop = threading.Event()
        self._proc = None

    def __enter__(self):
        q = ("clocks.sm,clocks.max.sm,clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
             "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")
        cmd = ["nvidia-smi", f"--query-gpu={q}", "--format=csv,noheader,nounits", "-lms", "200"]
        if self.uuid:
            cmd += ["-i", self.uuid]
        try:
            self._proc = subprocess.Popen(cmd, stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            threading.Thread(target=self._read, daemon=True).start()
        except OSError:
            self._proc = None
        return self

    def _read(self):
        for line in self._proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 6:
                self.samples.append(parts)

    def __exit__(self, *exc):
        if self._proc:
            time.sleep(0.25)
            self._proc.terminate()
            try:
                self._proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self._proc.kill()

    def summary(self):
        if not self.samples:
            return None
        sm = [float(s[0]) for s in self.samples if s[0].replace(".", "").isdigit()]
        mx = [float(s[1]) for s in self.samples if s[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for s in self.samples for i in range(4) if s[2 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": reasons, "samples": len(self.samples)}


def _cfg(name):
    from rtc8_gb300.configs import C1, C2, C5, C_ROOM
    return {"c1": C1, "c2": C2, "c5": C5, "room": C_ROOM}[name]


def _mlp_tensor_pipe():
    """Tensor-pipe utilisation of the MLP kernels recorded from an ncu capture in profiles/*.md
    (lines `tensor_pipe_active[<kernel>]: <percent of peak, elapsed cycles>`)."""
    out = {}
    pat = re.compile(r"tensor_pipe_active\[(\w+)\]:\s*([0-9.]+)")
    for f in sorted((ROOT / "profiles").glob("*.md")):
        for k, v in pat.findall(f.read_text()):
            out[k] = {"pct_of_peak": float(v), "source": f.name}
    return out


def _config_dict(cfg, world: int, active_leaves: int, total_leaves: int) -> dict:
    """The workload description both arms print (the same dict for the GPU arm and the CPU arm)."""
    return {"workload": _workload_name(cfg), "spp_per_step": STEP_SPP,
            "l2": f"GPU arm: flushed between steps ({L2_FLUSH_BYTES >> 20} MB write); CPU arm: not applicable",
            "active_leaves": int(active_leaves), "total_leaves": int(total_leaves),
            "parallelism": f"replicas x{world}"}


def _workload_name(cfg):
    v = cfg.volume
    return (f"{cfg.name}: plain volumetric path tracing, {cfg.width}x{cfg.height}, {STEP_SPP} spp per step, "
            f"fBm {v.n}^3{' (two clouds unioned)' if v.union_seed is not None else ''} "
            f"({'sparse, threshold ' + str(v.threshold) if v.threshold > 0 else 'dense'}), "
            f"sigma_t max {v.sigma_t_max}, albedo {cfg.albedo}, HG g {cfg.phase_param}, <= {cfg.max_bounces} bounces, "
            f"sun {cfg.sun_elevation_deg} deg + {'Hosek-Wilkie sky' if cfg.sky else 'constant env'}")


# ------------------------------------------------------------------------------ CPU legs
def cpu_sample(cfg, vox: np.ndarray, env_rgb: np.ndarray | None, target_seconds: float = 12.0, threads: int = 0):
    """Times the oracle (all host threads) on a bounded sample of the workload: bands of image rows
    spread over the frame, one sample per pixel per pass, passes repeated (sample 0, 1, ...) until
    about `target_seconds` of CPU work."""
    from oracle import orc

    threads = threads or (os.cpu_count() or 1)
    sc = orc.scene_from_config(cfg, vox, env_rgb)
    rng = orc.seed_states(cfg.width, cfg.height, cfg.rng_seed)
    # Bands of `threads` rows (one row per OpenMP thread) in bit-reversed order over the frame.
    band = threads
    nbands = max(1, cfg.height // band)
    bits = max(1, (nbands - 1).bit_length())
    order = sorted(range(nbands), key=lambda b: int(format(b, f"0{bits}b")[::-1], 2))
    paths = 0
    elapsed = 0.0
    passes = 0
    while elapsed < target_seconds:
        for b in order:
            if elapsed >= target_seconds:
                break
            y0 = b * band
            y1 = min(cfg.height, y0 + band)
            t0 = time.perf_counter()
            orc.render_plain(sc, rng, 1, accum_base=passes, rows=(y0, y1), threads=threads)
            elapsed += time.perf_counter() - t0
            paths += (y1 - y0) * cfg.width
        passes += 1
    return {"value": paths / elapsed, "unit": "paths/s", "cores": threads, "kind": "port",
            "sample": f"{paths} paths of {cfg.name} ({passes} pass(es) of 1 spp over row bands spread over the "
                      f"frame, {elapsed:.1f} s), oracle restatement with OpenMP"}


def scene_host_inputs(cfg):
    """Dense volume and environment image of a configuration for the CPU legs, built on the host
    by the oracle: its fBm generator (bit-identical to the device generator) and its float64
    restatement of the Hosek-Wilkie sky texture. No product library is loaded."""
    from oracle import orc
    from oracle import sky as osky
    from rtc8_gb300 import sky as psky
    from rtc8_gb300.configs import sun_direction

    vox = orc.fbm_volume(cfg.volume)
    env = None
    if cfg.sky is not None:
        d = sun_direction(cfg.sun_elevation_deg, cfg.sun_azimuth_deg).astype(np.float32)
        st = psky.load_sky_state(cfg.sky, cfg.sun_elevation_deg, d)
        env = osky.sky_texture(cfg.sky.width, cfg.sky.height, st["states"], st["cmf"], d).astype(np.float32)
    elif cfg.env_constant is not None:
        env = np.full((32, 64, 3), cfg.env_constant, dtype=np.float32)
    return vox, env


def leaf_counts(vox: np.ndarray) -> tuple[int, int]:
    """Non-empty and total 8^3 leaves of a dense volume."""
    lx, ly, lz = [(d + 7) // 8 for d in vox.shape]
    pad = np.zeros((lx * 8, ly * 8, lz * 8), np.float32)
    pad[:vox.shape[0], :vox.shape[1], :vox.shape[2]] = vox
    active = pad.reshape(lx, 8, ly, 8, lz, 8).max(axis=(1, 3, 5)) > 0
    return int(active.sum()), lx * ly * lz


def reference_arm(args, cfg, world: int) -> dict:
    """The CPU arm: the oracle's plain tracer (the reference's per-path algorithm restated in
    host C++, OpenMP over image rows, all host threads) on whole frames of the workload, STEP_SPP
    samples per pixel per step, timed step by step with the host clock."""
    from oracle import orc

    t_setup = time.perf_counter()
    vox, env = scene_host_inputs(cfg)
    active, total = leaf_counts(vox)
    sc = orc.scene_from_config(cfg, vox, env)
    del vox
    rng = orc.seed_states(cfg.width, cfg.height, cfg.rng_seed)
    sum_rgb = np.zeros((cfg.height, cfg.width, 3), dtype=np.float64)
    mean_rgb = np.zeros((cfg.height, cfg.width, 3), dtype=np.float32)
    threads = os.cpu_count() or 1
    setup_s = time.perf_counter() - t_setup
    step_s = []
    for i in range(args.warmup + args.steps):
        t0 = time.perf_counter()
        orc.render_plain(sc, rng, STEP_SPP, accum_base=i * STEP_SPP, threads=threads, sum_rgb=sum_rgb,
                         mean_rgb=mean_rgb)
        step_s.append(time.perf_counter() - t0)
    timed = step_s[args.warmup:] or step_s[-1:]
    ms = 1000.0 * sum(timed) / len(timed)
    paths = cfg.width * cfg.height * STEP_SPP
    value = paths / (ms / 1000.0)
    sample = (f"{len(timed)} timed frames of {cfg.width}x{cfg.height} x {STEP_SPP} spp of {cfg.name} after "
              f"{args.warmup} untimed ones, oracle restatement with OpenMP; inputs built on the host by the "
              f"oracle in {setup_s:.1f} s")
    return {"impl": "reference", "metric": "paths/s (plain volumetric path tracing)", "value": value,
            "unit": "paths/s", "n_gpus": world, "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms,
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (seeded fBm volume and Hosek-Wilkie sky built on the host)",
            "config": _config_dict(cfg, world, active, total),
            "cpu_baseline": {"value": value, "unit": "paths/s", "cores": threads, "kind": "port", "sample": sample},
            "e2e": {"value": value, "unit": "paths/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
            "gpu_launches": 0}


def mlp_bench(steps: int, warmup: int) -> dict:
    """The cache's MLP kernels alone at the sizes of a radiance-cache frame of the equal-error
    comparison: inference over 256^2 pixels x spp_per_frame queries (2^23 at 128 samples per frame)
    and training steps of 16384 records, volume encoding, 5 hidden layers of 64. FLOPs are those of
    the padded network (144x64 + 4x64x64 + 64x16 multiply-adds per record forward, 3x that per
    training record)."""
    import torch

    from rtc8_gb300 import convergence, nrc

    cfg = nrc.default_config(nrc.NRC_ENCODING_VOLUME)
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=cfg)
    gen = torch.Generator(device="cuda").manual_seed(0)
    n_inf, n_tr = 65536 * convergence.NRC_SETTINGS["spp_per_frame"], 16384
    q = torch.rand((n_inf, 14), device="cuda", generator=gen)
    q[:, 3:7] *= 3.0
    out = torch.empty((n_inf, 3), device="cuda")
    tgt = torch.rand((n_tr, 3), device="cuda", generator=gen)
    s = torch.cuda.current_stream()

    def timed(fn, n):
        for _ in range(warmup):
            fn()
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(n):
            fn()
        e.record(s)
        e.synchronize()
        return a.elapsed_time(e) / n / 1e3

    flop_fwd = 2 * (144 * 64 + 4 * 64 * 64 + 64 * 16)
    t_inf = timed(lambda: cache.infer(s.cuda_stream, q, n_inf, out), max(steps, 10))
    t_tr = timed(lambda: cache.train(s.cuda_stream, q, tgt, n_tr), max(steps, 10))
    # The training kernel at larger batches (one 128-record tile per CTA), to tell the kernel's
    # capability from the latency bound of the frame's 16384-record steps.
    big = {}
    for nb in (65536, 262144):
        tgt_b = torch.rand((nb, 3), device="cuda", generator=gen)
        t_b = timed(lambda: cache.train(s.cuda_stream, q, tgt_b, nb), 10)
        big[str(nb)] = {"train_step_ms": t_b * 1e3, "train_tflops": nb * 3 * flop_fwd / t_b / 1e12}
    peaks = json.loads((ROOT / "MEASURED_PEAKS.json").read_text()) if (ROOT / "MEASURED_PEAKS.json").exists() else {}
    peak = float(peaks.get("bf16_tflops", 1900.0))
    inf_tf = n_inf * flop_fwd / t_inf / 1e12
    # Ceiling of the network's MMA shapes: cycles per back-to-back M = 128, K = 16 MMA issued by one
    # thread at N = 16 (output layer), 64 (hidden and input layers) and 256 (the full rate). A
    # 128-row tile is 9 + 16 MMAs of N = 64 and 4 of N = 16; at the full rate its arithmetic would
    # take 128 * flop_fwd / 2 MACs / (MACs per cycle at N = 256).
    cyc = {str(nn): nrc.selftest_mma_rate(nn, 1024) for nn in (16, 64, 128, 256)}
    full_rate = 128 * 256 * 16 / cyc["256"]
    tile_floor = 25 * cyc["64"] + 4 * cyc["16"]
    mma_ceiling = {"cycles_per_mma": cyc, "tile_floor_cycles": tile_floor,
                   "tile_arith_cycles_at_full_rate": 128 * flop_fwd / 2 / full_rate,
                   "tensor_pipe_ceiling": 128 * flop_fwd / 2 / full_rate / tile_floor}
    tr_tf = n_tr * 3 * flop_fwd / t_tr / 1e12
    errors = cache.device_errors()
    cache.finalize()
    # The reference's own network (its initialize(HashGrid, 2, 0.01f) call): 16 hash-grid levels
    # of 2 features gathered and interpolated into the first layer's tile, OneBlob(4) angles and
    # identity reflectances (64 inputs), 2 hidden layers, output None; 2^23 queries and
    # 16384-record training steps (the tables' scatter-add and their Adam step included).
    hg = nrc.NeuralRadianceCache()
    hg.initialize(config=nrc.default_config(nrc.NRC_ENCODING_HASHGRID))
    flop_hg = 2 * (64 * 64 + 64 * 64 + 64 * 16)
    t_hi = timed(lambda: hg.infer(s.cuda_stream, q, n_inf, out), max(steps, 10))
    t_ht = timed(lambda: hg.train(s.cuda_stream, q, tgt, n_tr), max(steps, 10))
    hashgrid = {"infer_ms": t_hi * 1e3, "infer_queries_per_s": n_inf / t_hi,
                "infer_mlp_tflops": n_inf * flop_hg / t_hi / 1e12, "train_step_ms": t_ht * 1e3,
                "train_records_per_s": n_tr / t_ht, "device_errors": hg.device_errors()}
    hg.finalize()
    return {"metric": "MLP TFLOP/s (padded FP16 network, FP32 accumulation)", "infer_ms": t_inf * 1e3,
            "infer_tflops": inf_tf, "infer_frac_of_peak": inf_tf / peak, "train_step_ms": t_tr * 1e3,
            "train_tflops": tr_tf, "train_frac_of_peak": tr_tf / peak,
            "peak_tflops": peak, "peak_source": "measured bf16_tflops (dense FP16 has the same rate)",
            "infer_records": n_inf, "train_records": n_tr, "train_larger_batches": big,
            "mma_shape_ceiling": mma_ceiling, "hashgrid_reference_network": hashgrid, "device_errors": errors}


def nrc_frame_loop(frames: int, warmup: int, combined: bool = True) -> dict:
    """The radiance-cache frame loop (train_iterations training iterations + spp_per_frame samples
    per frame, the settings of the equal-error comparison) on the 256x256 dense 64^3 scene; returns
    the mean frame time."""
    import torch

    from rtc8_gb300 import convergence, nrc
    from rtc8_gb300.configs import C1
    from rtc8_gb300.renderer import Renderer, setup_scene

    st = convergence.NRC_SETTINGS
    r = Renderer(C1.width, C1.height)
    setup_scene(r, C1)
    r.nrc_set_query_density(True)
    r.nrc_set_termination_factor(st["termination"], st.get("train_termination", 0.0))
    r.nrc_set_combined_pass(combined)
    net = nrc.default_config(nrc.NRC_ENCODING_VOLUME)
    net.ema_decay, net.learning_rate = st["ema_decay"], st["learning_rate"]
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=net)
    s = torch.cuda.Stream()
    r.nrc_frame(cache, 8, st["spp_per_frame"], True, s.cuda_stream)
    iters = st.get("train_iterations", 1)
    for _ in range(warmup):
        r.nrc_frame(cache, iters, st["spp_per_frame"], False, s.cuda_stream)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(frames):
        r.nrc_frame(cache, iters, st["spp_per_frame"], False, s.cuda_stream)
    b.record(s)
    torch.cuda.synchronize()
    out = {"nrc_frame_ms": a.elapsed_time(b) / frames, "frames": frames, "spp_per_frame": st["spp_per_frame"],
           "train_iterations_per_frame": iters, "combined_pass": combined,
           "device_errors": r.device_errors() | cache.device_errors()}
    cache.finalize()
    r.close()
    return out


def nrc_equal_error_large(name: str) -> dict:
    """The radiance cache against the plain tracer to relMSE 1e-3 (held for 3 evaluations) on a
    large scene at full resolution, one seed: 16384-spp FP64 oracle image, plain in chunks of 64 spp,
    the cache with the comparison's settings at 32 samples per pixel per frame (the render pass
    keeps one query record per sample: 32 x 2048^2 records are 7.5 GB), error evaluated every 2nd
    frame."""
    from rtc8_gb300 import convergence

    cfg = _cfg(name)
    t0 = time.perf_counter()
    res = convergence.compare(cfg, target=1e-3, oracle_spp=16384, time_budget=1200.0, seeds=1,
                              settings={"spp_per_frame": 32}, plain_chunk=64, eval_every=2)
    out = {k: v for k, v in res.items() if k != "curves"}
    out["workload"] = _workload_name(cfg)
    out["wall_s"] = time.perf_counter() - t0
    out["curves"] = {k: [(int(a), round(b, 4), c) for a, b, c in v] for k, v in res["curves"].items()}
    return out


def nrc_equal_error_room() -> dict:
    """The radiance cache against the plain tracer to relMSE 1e-3 (held for 3 evaluations) on the
    mixed scene (the room's meshes around the 64^3 cloud) at 256^2, one seed: 16384-spp FP64 oracle
    image, plain in chunks of 16 spp, the cache with the reference's query encoding of surface
    vertices (the hash grid of its `initialize(HashGrid, 2, 0.01f)` call: 2 hidden layers) and
    the comparison's frame settings; repeated with the reference's own training settings (Adam lr
    1e-2, weight EMA 0.99) and with its path-termination factor (0.01)."""
    from rtc8_gb300 import convergence, nrc

    cfg = _cfg("room").replace(name="room_cloud64_256px", width=256, height=256)
    hg = {"encoding": nrc.NRC_ENCODING_HASHGRID}
    t0 = time.perf_counter()
    res = convergence.compare(cfg, target=1e-3, oracle_spp=16384, time_budget=120.0, seeds=1, settings=hg,
                              extra_settings={"reference_training": dict(hg, ema_decay=0.99, learning_rate=1e-2),
                                              "reference_termination": dict(hg, termination=0.01,
                                                                            train_termination=0.02)})
    out = {k: v for k, v in res.items() if k != "curves"}
    out["workload"] = f"{cfg.name}: room of 36 triangles (Lambert walls, two SimplePBR blocks, a rectangle light) around the 64^3 cloud, 256x256"
    out["wall_s"] = time.perf_counter() - t0
    return out


def stress_plain(steps: int = 3, warmup: int = 2) -> dict:
    """The plain tracer on the 2048^2 stress scene (1024^3, two unioned fBm clouds, sigma_t max 400,
    albedo 0.9995, g 0.9, <= 1024 bounces), STEP_SPP per launch, device-timed."""
    import torch

    from rtc8_gb300.configs import C5
    from rtc8_gb300.renderer import Renderer, setup_scene

    r = Renderer(C5.width, C5.height)
    setup_scene(r, C5)
    s = torch.cuda.current_stream()
    for _ in range(warmup):
        r.launch_plain(STEP_SPP, s.cuda_stream)
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(steps):
        r.launch_plain(STEP_SPP, s.cuda_stream)
    b.record(s)
    b.synchronize()
    ms = a.elapsed_time(b) / steps
    info = r.volume_info()
    out = {"workload": _workload_name(C5), "ms_per_launch": ms,
           "paths_per_s": C5.width * C5.height * STEP_SPP / (ms / 1e3), "launches": steps,
           "active_leaves": info["active_leaves"], "total_leaves": info["total_leaves"],
           "device_errors": r.device_errors()}
    r.close()
    return out


def surface_plain(steps: int = 3, warmup: int = 2, cfg_name: str = "room_cloud64_512px") -> dict:
    """The surface tracer on the mixed scene (the 64^3 cloud inside an open room of Lambert walls,
    two SimplePBR blocks and a rectangle light, 512^2), STEP_SPP per launch, device-timed; with the
    room's BVH and emitter counts and the work counters (lookups per path)."""
    import torch

    from rtc8_gb300.configs import CONFIGS
    from rtc8_gb300.renderer import Renderer, setup_scene

    cfg = CONFIGS[cfg_name]
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg)
    s = torch.cuda.current_stream()
    for _ in range(warmup):
        r.launch_plain(STEP_SPP, s.cuda_stream)
    torch.cuda.synchronize()
    r.reset_counters()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(s)
    for _ in range(steps):
        r.launch_plain(STEP_SPP, s.cuda_stream)
    b.record(s)
    b.synchronize()
    ms = a.elapsed_time(b) / steps
    c = r.counters()
    out = {"workload": f"{cfg.name}: {cfg.width}x{cfg.height}, {STEP_SPP} spp per launch, fBm {cfg.volume.n}^3 "
                       f"cloud in a room of {r.surface_info()['triangles']} triangles (Lambert walls, SimplePBR "
                       "blocks, rectangle light), sun + constant environment through the open side",
           "ms_per_launch": ms, "paths_per_s": cfg.width * cfg.height * STEP_SPP / (ms / 1e3), "launches": steps,
           "surfaces": r.surface_info(), "vertices_per_path": c["vertices"] / max(c["samples"], 1),
           "lookups_per_path": c["lookups"] / max(c["samples"], 1), "device_errors": r.device_errors()}
    r.close()
    return out


def batch_bench(steps: int, warmup: int, spp: int = 4) -> dict:
    """The batched workload: 16 seeded scenes of uneven resolution and grid size, one batch
    step = `spp` samples per pixel of every scene as one CUDA-graph launch, launch shapes picked by
    the autotuner; the same step issued launch by launch is timed for comparison."""
    import torch

    from rtc8_gb300.batch import SceneBatch, make_c4_scenes

    b = SceneBatch(make_c4_scenes(16, 4))
    tuned = b.autotune(spp=2)
    b.capture(spp)
    s = torch.cuda.current_stream()

    def timed(fn, n):
        a, e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        a.record(s)
        for _ in range(n):
            fn()
        e.record(s)
        e.synchronize()
        return a.elapsed_time(e) / n

    for _ in range(warmup):
        b.step()
    graph_ms = timed(b.step, steps)
    for _ in range(warmup):
        b.step_uncaptured(spp)
    plain_ms = timed(lambda: b.step_uncaptured(spp), steps)
    paths = b.paths_per_step
    errors = sum(r.device_errors() for r in b.renderers)
    # The radiance-cache form: every scene with its own cache, one frame of every scene per step.
    b.enable_caches()
    b.nrc_step(spp, train_iterations=8, new_sequence=True)
    for _ in range(warmup):
        b.nrc_step(spp)
    nrc_ms = timed(lambda: b.nrc_step(spp), steps)
    nrc = {"ms_per_step": nrc_ms, "paths_per_s": paths / (nrc_ms / 1e3), "spp_per_scene": spp,
           "train_iterations_per_frame": b.nrc_settings.get("train_iterations", 1),
           "training_records_per_frame": 4 * 16384 * b.nrc_settings.get("train_iterations", 1),
           "device_errors": b.nrc_errors(),
           "form": "per-scene caches, each scene's frame on its own stream (not graph-captured: the frame "
                   "draws its unbiased-path offsets on the host)"}
    out = {"metric": "paths/s (16 batched scenes, one CUDA graph per step)", "value": paths / (graph_ms / 1e3),
           "unit": "paths/s", "n_gpus": 1, "steps": steps, "warmup": warmup, "ms_per_step": graph_ms,
           "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
           "data": "synthetic (seeded fBm volumes generated on the device)",
           "config": {"workload": f"c4: 16 scenes, {spp} spp per scene per step, {paths} paths per step",
                      "scenes": [{"name": c.name, "g": round(c.phase_param, 3), **{k: v for k, v in t.items()
                                                                                   if k != "scene"}}
                                 for c, t in zip(b.configs, tuned)]},
           "uncaptured_ms_per_step": plain_ms, "device_errors": errors, "nrc": nrc}
    b.close()
    return out


# ------------------------------------------------------------------------------ main
def max_over_ranks(ms: float, world: int, device) -> float:
    """The slowest rank's time for the same timed region (every rank passed a barrier before it):
    whole-job throughput is the units all ranks processed divided by this time."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist

    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=4)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--config", default="c2", choices=["c1", "c2", "c4", "c5", "room"])
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--image", type=int, default=0, help="override the image side (profiling runs)")
    ap.add_argument("--no-flush", action="store_true", help="skip the L2 flush between steps (profiling runs)")
    ap.add_argument("--no-nrc", action="store_true", help="skip the NRC-vs-plain equal-error comparison")
    ap.add_argument("--no-mlp", action="store_true", help="skip the MLP kernel figures of the default line")
    ap.add_argument("--tracker", default="megakernel", choices=["megakernel", "wavefront"],
                    help="plain tracker: the persistent megakernel (default) or the wavefront form")
    ap.add_argument("--mlp", action="store_true",
                    help="profiling run: only the cache's MLP kernels (inference and training steps)")
    ap.add_argument("--nrc-frames", type=int, default=0,
                    help="profiling run: only the radiance-cache frame loop on the 256x256 scene, N timed frames")
    ap.add_argument("--nrc-equal-error", default="", choices=["", "c5", "c2", "room"],
                    help="only the radiance-cache vs plain equal-error comparison on the 2048^2 stress scene (c5), "
                         "the 1024^2 sparse scene (c2) or the mixed surface scene at 256^2 (room), one seed")
    ap.add_argument("--nrc-separate-passes", action="store_true",
                    help="with --nrc-frames: first training pass and render samples as two launches")
    ap.add_argument("--leaf-stage", type=int, default=0,
                    help="per-warp leaf staging in shared memory when this many lanes share a leaf (0 = off)")
    ap.add_argument("--no-extras", action="store_true",
                    help="skip the stress-scene and batched-scene figures of the default line")
    args = ap.parse_args()
    warmup = max(args.warmup, 3)

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if args.impl == "reference":
        # Rank 0 alone runs the CPU arm; it needs neither a GPU nor a process group.
        if rank == 0:
            print(json.dumps(reference_arm(args, _cfg(args.config if args.config != "c4" else "c2"), world)),
                  flush=True)
        return

    import torch
    import torch.distributed as dist

    if world > 1:
        dist.init_process_group("nccl")
    if args.config == "c4" and args.impl == "ours":
        if rank == 0:
            torch.cuda.set_device(local)
            print(json.dumps(batch_bench(args.steps, warmup)), flush=True)
        return
    cfg = _cfg(args.config if args.config != "c4" else "c1")
    if args.image:
        cfg = cfg.replace(width=args.image, height=args.image)

    from rtc8_gb300.renderer import Renderer, setup_scene

    if args.mlp:
        torch.cuda.set_device(local)
        print(json.dumps(mlp_bench(args.steps, warmup)), flush=True)
        return
    if args.nrc_frames:
        torch.cuda.set_device(local)
        print(json.dumps(nrc_frame_loop(args.nrc_frames, warmup, not args.nrc_separate_passes)), flush=True)
        return
    if args.nrc_equal_error:
        torch.cuda.set_device(local)
        res = nrc_equal_error_room() if args.nrc_equal_error == "room" else nrc_equal_error_large(args.nrc_equal_error)
        print(json.dumps(res), flush=True)
        return

    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg)
    r.set_tracker(1 if args.tracker == "wavefront" else 0)
    r.set_leaf_staging(args.leaf_stage)
    info = r.volume_info()
    stream = torch.cuda.Stream(device=dev)
    sptr = stream.cuda_stream
    flush = None if args.no_flush else torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    pinned = torch.empty(cfg.height * cfg.width * 3, dtype=torch.float32, pin_memory=True)

    def flush_l2():
        with torch.cuda.stream(stream):
            if flush is not None:
                flush.fill_(1.0)

    # ---- device-timed steps (inputs resident in HBM)
    for _ in range(warmup):
        flush_l2()
        r.launch_plain(STEP_SPP, sptr)
    torch.cuda.synchronize()
    r.reset_counters()
    if world > 1:
        dist.barrier()
    torch.cuda.synchronize()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(args.steps)]
    uuid = None
    try:
        uuid = str(torch.cuda.get_device_properties(dev).uuid)
        uuid = uuid if uuid.startswith("GPU-") else "GPU-" + uuid
    except Exception:
        uuid = None
    with ClockSampler(uuid) as clk:
        for i in range(args.steps):
            flush_l2()
            ev[i][0].record(stream)
            r.launch_plain(STEP_SPP, sptr)
            ev[i][1].record(stream)
        torch.cuda.synchronize()
    step_ms = [a.elapsed_time(b) for a, b in ev]
    cnt = r.counters()
    total_ms = max_over_ranks(float(sum(step_ms)), world, dev)
    paths_per_rank = cfg.width * cfg.height * STEP_SPP * args.steps
    value = world * paths_per_rank / (total_ms / 1000.0)

    # ---- end to end through the C ABI with host buffers (result image read back every step)
    lib = r.lib
    import ctypes as C
    e2e_ms = []
    d2h = cfg.height * cfg.width * 3 * 4
    h2d = C.sizeof(r.params)
    for i in range(warmup + args.steps):
        flush_l2()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        r.set_frame(r.params)                   # per-frame parameters from the host
        r.launch_plain(STEP_SPP, sptr)
        lib.vpt_download_mean(r.ctx, C.cast(pinned.data_ptr(), C.POINTER(C.c_float)))
        t1 = time.perf_counter()
        if i >= warmup:
            e2e_ms.append(1000.0 * (t1 - t0))
    if world > 1:
        dist.barrier()
    e2e_total = max_over_ranks(sum(e2e_ms), world, dev)
    e2e_value = world * paths_per_rank / (e2e_total / 1000.0)

    # ---- roofline of the tracer kernel (algorithmic bytes per launch / average launch time).
    # Algorithmic unit of the tracking work: 32 B per density lookup (the 2x2x2 FP32 stencil),
    # 120 B per path vertex (path state read and written once per vertex) and 48 B per sample
    # (FP64 RGB accumulator read and written); lookups, vertices and samples from device counters.
    lookups_per_launch = cnt["lookups"] / args.steps
    vertices_per_launch = cnt["vertices"] / args.steps
    samples_per_launch = cnt["samples"] / args.steps
    alg_bytes = 32.0 * lookups_per_launch + 120.0 * vertices_per_launch + 48.0 * samples_per_launch
    launch_s = total_ms / args.steps / 1000.0
    achieved = alg_bytes / launch_s / 1e9
    pixels = cfg.width * cfg.height
    # The persistent tracker keeps path state in registers, so the bytes it must move are fewer:
    reg_bytes = 32.0 * lookups_per_launch + 88.0 * pixels
    peak, peak_kind = _peaks()
    traffic, prof = _profile_traffic("plain_trace_kernel", args.config)
    roofline = {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                "traffic": traffic, "peak_source": f"{peak_kind} hbm_gbs", "traffic_source": prof,
                "algorithmic_bytes_per_launch": alg_bytes,
                "algorithmic_unit": "32 B x lookups + 120 B x path vertices + 48 B x samples",
                "lookups_per_launch": lookups_per_launch, "vertices_per_launch": vertices_per_launch,
                "samples_per_launch": samples_per_launch,
                "register_resident_state": {"bytes_per_launch": reg_bytes,
                                            "achieved": reg_bytes / launch_s / 1e9,
                                            "frac": reg_bytes / launch_s / 1e9 / peak,
                                            "unit": "32 B x lookups + 88 B x pixels (PCG state, FP64 sum, "
                                                    "FP32 mean)"}}

    # ---- radiance cache vs plain at equal error (NRC form of the 256x256 dense 64^3 configuration)
    nrc_cmp = None
    if rank == 0 and not args.no_nrc:
        from rtc8_gb300 import convergence
        from rtc8_gb300.configs import C1
        res = convergence.compare(C1, target=1e-3, oracle_spp=16384, time_budget=60.0, seeds=3,
                                  extra_settings={"adam_lr_1e-2": {"learning_rate": 1e-2}})
        nrc_cmp = {k: v for k, v in res.items() if k != "curves"}
        nrc_cmp["workload"] = (f"{C1.name}: 256x256, dense fBm 64^3, sigma_t max {C1.volume.sigma_t_max}, "
                               f"albedo {C1.albedo}, HG g {C1.phase_param}, sun + constant env 0.5")
        nrc_cmp["time"] = ("seconds: GPU time of each estimator's launches (CUDA events); wall_seconds: host "
                           "wall clock around the same launches; error evaluation excluded from both")

    mlp = None
    if rank == 0 and not args.no_mlp:
        mlp = mlp_bench(10, warmup)
        mlp["tensor_pipe_ncu"] = _mlp_tensor_pipe()

    extras = None
    if rank == 0 and not args.no_extras and args.config == "c2":
        extras = {}
        for key, fn in (("stress_2048px_1024cube_plain", lambda: stress_plain()),
                        ("room_512px_surfaces_cloud64", lambda: surface_plain()),
                        ("batched_16_scenes", lambda: batch_bench(3, 2))):
            try:
                extras[key] = fn()
            except Exception as e:  # reported in the line; the headline measurement stands
                extras[key] = {"error": f"{type(e).__name__}: {e}"}
            torch.cuda.empty_cache()

    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        vox, env = scene_host_inputs(cfg)
        cpu = cpu_sample(cfg, vox, env, target_seconds=12.0)
        del vox

    if rank == 0:
        line = {"metric": "paths/s (plain volumetric path tracing)", "value": value, "unit": "paths/s",
                "n_gpus": world, "steps": args.steps, "warmup": warmup, "ms_per_step": total_ms / args.steps,
                "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (seeded fBm volume generated on the device)",
                "config": _config_dict(cfg, world, info["active_leaves"], info["total_leaves"]),
                "e2e": {"value": e2e_value, "unit": "paths/s", "h2d_bytes_per_step": h2d,
                        "d2h_bytes_per_step": d2h},
                "gpu_launches": args.steps * (3 if cfg.rng_stream_mode == 1 else 1),  # jump table, tracer, mean
                "nrc_vs_plain": nrc_cmp,
                "mlp": mlp,
                "other_workloads": extras,
                "roofline": roofline,
                "cpu_baseline": cpu,
                "clocks": clk.summary(),
                "counters": cnt,
                "device_errors": r.device_errors()}
        print(json.dumps(line), flush=True)
    r.close()
    if world > 1:
        dist.destroy_process_group()


if __name__ == "__main__":
    main()
