"""Equal-error comparison of the radiance-cache renderer with the plain path tracer.

Both estimators render the same scene; after every chunk of work the accumulated image is
compared with an FP64-accumulated high-spp image of the plain tracer made from independent
RNG streams (the "oracle image"). The error measure is the relative MSE

    relMSE = mean over pixels and channels of (x - ref)^2 / (ref^2 + 0.01)

(the 0.01 keeps dark pixels from dominating). Time is GPU time of the estimator's own launches
(CUDA events on its stream) and, next to it, the host wall clock around the same launches, both
excluding the error evaluation. An estimator has reached the target when the error stays at or
below it for `SUSTAIN` consecutive evaluations; its time is the time of the first of them. The
comparison runs several independent RNG seeds and reports the median. The radiance-cache estimator runs
the reference's frame loop (renderer/renderer_main.cpp:1553-1637): every frame trains the cache
on that frame's training suffixes and renders `spp_per_frame` samples per pixel (batched into one
render pass on sample-parallel streams); the first frame trains eight times (a new sequence).
"""
from __future__ import annotations

import math
import time

import numpy as np

from .configs import SceneConfig
from .renderer import Renderer, setup_scene

REL_EPS = 1e-2
SUSTAIN = 3


def rel_mse(img, ref) -> float:
    import torch

    a = torch.as_tensor(img, dtype=torch.float64)
    b = torch.as_tensor(ref, dtype=torch.float64)
    return float(((a - b) ** 2 / (b * b + REL_EPS)).mean())


def oracle_image(cfg: SceneConfig, spp: int, seed_offset: int = 1, chunk: int = 256, stream=None) -> np.ndarray:
    """FP64-accumulated plain image with `spp` samples per pixel from RNG streams independent of
    the configuration's own (seed + seed_offset)."""
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg)
    r.seed_rng(cfg.rng_seed + seed_offset)
    done = 0
    while done < spp:
        n = min(chunk, spp - done)
        r.launch_plain(n, stream)
        done += n
    r.synchronize(stream)
    img = r.image()
    r.close()
    return img


def _timed(stream, fn) -> tuple[float, float]:
    """(GPU seconds between events around `fn` on `stream`, host wall seconds until they completed)."""
    import torch

    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    t0 = time.perf_counter()
    a.record(stream)
    fn()
    b.record(stream)
    b.synchronize()
    wall = time.perf_counter() - t0
    return a.elapsed_time(b) / 1000.0, wall


class _Reach:
    """Tracks the first evaluation of a run of SUSTAIN consecutive evaluations at or below target."""

    def __init__(self, target: float, sustain: int = SUSTAIN):
        self.target, self.sustain = target, sustain
        self.first = None        # first evaluation at or below the target at all
        self.candidate = None    # start of the current run
        self.streak = 0
        self.reached = None

    def update(self, record: dict, error: float) -> bool:
        """Returns True once the target has held for `sustain` evaluations."""
        if error <= self.target:
            if self.first is None:
                self.first = dict(record)
            if self.streak == 0:
                self.candidate = dict(record)
            self.streak += 1
            if self.streak >= self.sustain and self.reached is None:
                self.reached = self.candidate
        else:
            self.streak = 0
            self.candidate = None
        return self.reached is not None


def plain_curve(cfg: SceneConfig, ref: np.ndarray, target: float, chunk_spp: int = 16, max_spp: int = 16384,
                time_budget: float = 60.0) -> dict:
    """relMSE of the plain tracer after each chunk of `chunk_spp` samples per pixel."""
    import torch

    s = torch.cuda.Stream()
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg)
    curve, t, wall, spp, img = [], 0.0, 0.0, 0, None
    reach = _Reach(target)
    wall0 = time.perf_counter()
    while spp < max_spp and time.perf_counter() - wall0 < time_budget:
        dt, dw = _timed(s, lambda: r.launch_plain(chunk_spp, s.cuda_stream))
        t, wall, spp = t + dt, wall + dw, spp + chunk_spp
        img = r.image()
        e = rel_mse(img, ref)
        curve.append((spp, t, e))
        if reach.update({"spp": spp, "seconds": t, "wall_seconds": wall}, e):
            break
    r.close()
    return {"curve": curve, "reached": reach.reached, "first_below": reach.first, "image": img}


def nrc_curve(cfg: SceneConfig, ref: np.ndarray, target: float, net_config=None, spp_per_frame: int = 8,
              eval_every: int = 1, max_frames: int = 4096, time_budget: float = 60.0,
              query_density: bool = True, termination: float = 0.0, warmup_frames: int = 0,
              train_termination: float = 0.0, train_iterations: int = 1, first_train_iterations: int = 8) -> dict:
    """relMSE of the radiance-cache renderer after every `eval_every` frames of `spp_per_frame`
    samples per pixel (the reference renders 8 samples per frame, renderer_main.cpp:359). The
    images of the first frame and of `warmup_frames` more frames (rendered while the cache is
    still young) are dropped from the accumulation; their time counts."""
    import torch

    from . import nrc

    s = torch.cuda.Stream()
    r = Renderer(cfg.width, cfg.height)
    setup_scene(r, cfg)
    r.nrc_set_query_density(query_density)
    r.nrc_set_termination_factor(termination, train_termination)
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=net_config or nrc.default_config(nrc.NRC_ENCODING_VOLUME))
    curve, img = [], None
    t, wall = _timed(s, lambda: r.nrc_frame(cache, first_train_iterations, spp_per_frame, True, s.cuda_stream))
    for _ in range(warmup_frames):
        dt, dw = _timed(s, lambda: r.nrc_frame(cache, 1, spp_per_frame, False, s.cuda_stream))
        t, wall = t + dt, wall + dw
    frames = 1 + warmup_frames
    if warmup_frames:
        r.reset_accumulation()
    reach = _Reach(target)
    wall0 = time.perf_counter()
    while frames < max_frames and time.perf_counter() - wall0 < time_budget:
        def run():
            for _ in range(eval_every):
                r.nrc_frame(cache, train_iterations, spp_per_frame, False, s.cuda_stream)
        dt, dw = _timed(s, run)
        t, wall, frames = t + dt, wall + dw, frames + eval_every
        img = r.image()
        e = rel_mse(img, ref)
        curve.append((frames * spp_per_frame, t, e))
        if reach.update({"frames": frames, "spp": frames * spp_per_frame, "seconds": t, "wall_seconds": wall}, e):
            break
    errors = r.device_errors() | cache.device_errors()
    best = min(c[2] for c in curve) if curve else math.inf
    r.close()
    cache.finalize()
    return {"curve": curve, "reached": reach.reached, "first_below": reach.first, "best_rel_mse": best,
            "device_errors": errors, "image": img}


# Radiance-cache settings of the equal-error comparison, from sweeps on the 64^3 cloud with RNG
# seeds that the comparison itself does not use, judged by the sustained criterion: the volume
# cache of rtc8_nrc.h with Adam lr 5e-3; 128 samples per pixel per frame with four training
# iterations (generate, propagate, shuffle, 4 x 16384-record steps) per frame and three in the
# first frame; render paths end at path-spread factor 0.9 and biased training suffixes at 0.08;
# inference with an EMA of the weights at decay 0.8. Sweeps on ten held-out seeds with the
# pixel-major sample order: first-frame iterations {5, 6, 7, 8} x render factor {0.9, 1.0, 1.1,
# 1.28} x decay {0.7, 0.8} gave a mean speed-up of 2.90 at (5, 0.9, 0.8) against 2.75 at the
# earlier (8, 1.28, 0.8); then, with 8 cells per tracking step, first-frame iterations 1 / 2 / 3 /
# 4 / 5 gave means 2.97 / 3.14 / 3.14 / 3.05 / 2.99 at factor 0.9 (factor 0.8: 3.18 at 2, 3.08 at
# 3); 96 / 112 / 160 spp per frame, 3 or 5 iterations per frame and decay 0.9 were slower. Render
# paths use the configuration's shadow-ray roulette; the training suffixes do not.
NRC_SETTINGS = {"termination": 0.9, "train_termination": 0.08, "ema_decay": 0.8, "learning_rate": 5e-3,
                "spp_per_frame": 128, "train_iterations": 4, "first_train_iterations": 3}


def compare_once(cfg: SceneConfig, ref: np.ndarray, target: float, st: dict, time_budget: float,
                 plain_chunk: int = 16, eval_every: int = 1) -> dict:
    """One equal-error comparison on `cfg` (its RNG seed) against the oracle image `ref`."""
    from . import nrc

    # The volume encoding by default; scenes with meshes take the reference's query encodings
    # (settings "encoding"), whose inputs hold the surface normal, roughness and reflectances.
    net = nrc.default_config(st.get("encoding", nrc.NRC_ENCODING_VOLUME))
    net.ema_decay = st["ema_decay"]
    net.learning_rate = st["learning_rate"]
    plain = plain_curve(cfg, ref, target, chunk_spp=plain_chunk, time_budget=time_budget)
    cache = nrc_curve(cfg, ref, target, net_config=net, spp_per_frame=st["spp_per_frame"], time_budget=time_budget,
                      termination=st["termination"], train_termination=st.get("train_termination", 0.0),
                      train_iterations=st.get("train_iterations", 1), eval_every=eval_every,
                      first_train_iterations=st.get("first_train_iterations", 8),
                      max_frames=max(16, 16384 // st["spp_per_frame"]))
    out = {"rng_seed": cfg.rng_seed,
           "plain": {"reached": plain["reached"], "first_below": plain["first_below"],
                     "last": plain["curve"][-1] if plain["curve"] else None},
           "nrc": {"reached": cache["reached"], "first_below": cache["first_below"],
                   "last": cache["curve"][-1] if cache["curve"] else None,
                   "best_rel_mse": cache["best_rel_mse"], "device_errors": cache["device_errors"]}}
    # MLP error: relMSE of the radiance-cache estimate against the plain estimate, both at the
    # point where they stopped.
    if cache["image"] is not None and plain["image"] is not None:
        out["nrc"]["mlp_error_vs_plain"] = rel_mse(cache["image"], plain["image"])
    if plain["reached"] and cache["reached"]:
        out["speedup"] = plain["reached"]["seconds"] / cache["reached"]["seconds"]
        out["speedup_wall"] = plain["reached"]["wall_seconds"] / cache["reached"]["wall_seconds"]
    else:
        out["speedup"] = out["speedup_wall"] = None
    out["curves"] = {"plain": plain["curve"], "nrc": cache["curve"]}
    return out


def _median(xs):
    xs = sorted(x for x in xs if x is not None)
    return xs[len(xs) // 2] if len(xs) % 2 else (0.5 * (xs[len(xs) // 2 - 1] + xs[len(xs) // 2]) if xs else None)


def compare(cfg: SceneConfig, target: float = 1e-3, oracle_spp: int = 16384, time_budget: float = 60.0,
            settings: dict | None = None, seeds: int = 3, extra_settings: dict | None = None,
            plain_chunk: int = 16, eval_every: int = 1) -> dict:
    """Time to reach relMSE <= target (held for SUSTAIN evaluations) for both estimators on `cfg`,
    for `seeds` independent RNG seeds of both estimators; the headline is the median speed-up.
    `extra_settings` ({name: overrides}) repeats the radiance-cache runs with other settings."""
    st = dict(NRC_SETTINGS, **(settings or {}))
    ref = oracle_image(cfg, oracle_spp)
    runs = [compare_once(cfg.replace(rng_seed=cfg.rng_seed + 7919 * (k + 1)), ref, target, st, time_budget,
                         plain_chunk, eval_every) for k in range(seeds)]
    out = {"target_rel_mse": target, "sustained_evaluations": SUSTAIN, "oracle_spp": oracle_spp,
           "rel_mse_eps": REL_EPS, "nrc_settings": st, "seeds": seeds,
           "speedup": _median([r["speedup"] for r in runs]),
           "speedup_wall": _median([r["speedup_wall"] for r in runs]),
           "speedups": [r["speedup"] for r in runs], "speedups_wall": [r["speedup_wall"] for r in runs],
           "plain_chunk_spp": plain_chunk, "nrc_eval_every_frames": eval_every,
           "runs": [{k: v for k, v in r.items() if k != "curves"} for r in runs]}
    for name, over in (extra_settings or {}).items():
        st2 = dict(st, **over)
        more = [compare_once(cfg.replace(rng_seed=cfg.rng_seed + 7919 * (k + 1)), ref, target, st2, time_budget)
                for k in range(seeds)]
        out[name] = {"nrc_settings": st2, "speedup": _median([r["speedup"] for r in more]),
                     "speedups": [r["speedup"] for r in more],
                     "speedups_wall": [r["speedup_wall"] for r in more],
                     "nrc_reached": [r["nrc"]["reached"] for r in more],
                     "mlp_error_vs_plain": [r["nrc"].get("mlp_error_vs_plain") for r in more]}
    out["curves"] = runs[0]["curves"]
    return out
