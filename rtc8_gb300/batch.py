"""Batched rendering of many independent scenes (16 scenes of uneven resolution and grid size).

Every scene keeps its own context (volume, environment, camera, image size, RNG streams and,
for the radiance-cache form, its own cache). One batch step renders `spp` samples per pixel of
every scene: the scenes' launches are issued on one stream each, forked from and joined back to
the caller's stream, and the whole step is captured once as a CUDA graph and replayed, so a step
costs one graph launch. The device frame counters of each context advance inside the graph, so
every replay renders new samples. Branches of the graph run concurrently, so one scene's launch
tail overlaps the next scene's work.

The autotuner picks per scene the tracker's launch shape (CTAs per SM and the warp park
threshold) by timing a short launch of each candidate.
"""
from __future__ import annotations

import math
import time

import numpy as np

from .configs import C1, SceneConfig, VolumeSpec
from .renderer import Renderer, setup_scene

# Launch shapes the autotuner tries: (CTAs per SM, park threshold); 0 = the defaults. The batch's
# launches run CTAs of 128 threads (BATCH_THREADS): alone, a scene's plain launch is fastest as one
# 896-thread CTA per SM, but the batch's concurrent launches then cannot share an SM (16 scenes:
# 606 M paths/s against 647 M with 128-thread CTAs).
LAUNCH_CANDIDATES = [(0, 0), (0, 16), (0, 28), (6, 24), (5, 24)]
BATCH_THREADS = 128


def make_c4_scenes(count: int = 16, seed: int = 4) -> list[SceneConfig]:
    """The batched workload's scenes: resolution from {256, 512, 768, 1024}^2, fBm grid from
    {64, 128, 256, 512}^3 (sparse above 64^3), HG g uniform in [0.3, 0.9], drawn from `seed`."""
    rng = np.random.default_rng(seed)
    out = []
    for i in range(count):
        res = int(rng.choice([256, 512, 768, 1024]))
        n = int(rng.choice([64, 128, 256, 512]))
        g = float(rng.uniform(0.3, 0.9))
        octaves = 4 + int(round(math.log2(n / 64)))
        vol = VolumeSpec(n=n, seed=100 + i, octaves=octaves, threshold=0.0 if n == 64 else 0.5,
                         sigma_t_max=20.0 * n / 64)
        out.append(C1.replace(name=f"c4_scene{i:02d}_{res}px_{n}cube", width=res, height=res, spp=16, volume=vol,
                              phase_param=g, majorant_cell_log2=max(3, int(math.log2(n)) - 4),
                              rng_seed=C1.rng_seed + i))
    return out


class SceneBatch:
    """Independent scenes rendered together; see the module docstring."""

    def __init__(self, configs: list[SceneConfig]):
        import torch

        self.configs = list(configs)
        self.renderers = []
        for cfg in self.configs:
            r = Renderer(cfg.width, cfg.height)
            setup_scene(r, cfg)
            # The batch step is one CUDA graph: its launches are the persistent megakernel (the
            # wavefront tracer issues its passes from the host and cannot be captured).
            r.set_tracker(0)
            r.set_launch_shape(0, BATCH_THREADS, 0)
            self.renderers.append(r)
        self.streams = [torch.cuda.Stream() for _ in self.renderers]
        self.graph = None
        self.graph_spp = 0
        self.shapes = [(0, 0)] * len(self.renderers)

    @property
    def paths_per_step(self) -> int:
        return sum(c.width * c.height for c in self.configs) * self.graph_spp

    def close(self) -> None:
        for c in getattr(self, "caches", []):
            c.finalize()
        self.caches = []
        for r in self.renderers:
            r.close()
        self.renderers = []
        self.graph = None

    # ------------------------------------------------------------------ autotuner
    def autotune(self, spp: int = 4, candidates=LAUNCH_CANDIDATES) -> list[dict]:
        """Times one launch of `spp` samples per candidate launch shape, per scene, keeps the
        fastest, and resets the accumulations."""
        import torch

        report = []
        for i, r in enumerate(self.renderers):
            s = self.streams[i]
            best = None
            for ctas, park in candidates:
                r.set_launch_shape(ctas, BATCH_THREADS, park)
                r.launch_plain(spp, s.cuda_stream)  # warm
                a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
                a.record(s)
                r.launch_plain(spp, s.cuda_stream)
                b.record(s)
                b.synchronize()
                ms = a.elapsed_time(b)
                if best is None or ms < best[0]:
                    best = (ms, ctas, park)
            r.set_launch_shape(best[1], BATCH_THREADS, best[2])
            r.reset_accumulation()
            self.shapes[i] = (best[1], best[2])
            report.append({"scene": self.configs[i].name, "ctas_per_sm": best[1], "park_threshold": best[2],
                           "ms_per_launch": best[0], "spp": spp})
        self.graph = None  # launch shapes are part of the captured launches
        return report

    # ------------------------------------------------------------------ graph
    def _issue(self, spp: int) -> None:
        import torch

        origin = torch.cuda.current_stream()
        for r, s in zip(self.renderers, self.streams):
            s.wait_stream(origin)
            r.launch_plain(spp, s.cuda_stream)
        for s in self.streams:
            origin.wait_stream(s)

    def capture(self, spp: int) -> None:
        """Captures one batch step of `spp` samples per pixel per scene as a CUDA graph."""
        import torch

        # Warm-up outside the capture: allocates the jump tables and builds the majorant grids.
        self._issue(spp)
        torch.cuda.synchronize()
        for r in self.renderers:
            r.reset_accumulation()
        g = torch.cuda.CUDAGraph()
        with torch.cuda.graph(g, capture_error_mode="thread_local"):
            self._issue(spp)
        torch.cuda.synchronize()
        self.graph = g
        self.graph_spp = spp

    def step(self) -> None:
        """One batch step (one graph launch)."""
        if self.graph is None:
            raise RuntimeError("capture() first")
        self.graph.replay()

    def step_uncaptured(self, spp: int) -> None:
        """The same step issued launch by launch (for comparison)."""
        self._issue(spp)

    # ------------------------------------------------------------------ radiance caches
    def enable_caches(self, settings: dict | None = None) -> None:
        """Gives every scene its own radiance cache (the volume network of rtc8_nrc.h) with the
        equal-error comparison's settings (rtc8_gb300.convergence.NRC_SETTINGS)."""
        from . import convergence, nrc

        st = dict(convergence.NRC_SETTINGS, **(settings or {}))
        self.nrc_settings = st
        self.caches = []
        for r in self.renderers:
            r.nrc_set_query_density(True)
            r.nrc_set_termination_factor(st["termination"], st.get("train_termination", 0.0))
            net = nrc.default_config(nrc.NRC_ENCODING_VOLUME)
            net.ema_decay, net.learning_rate = st["ema_decay"], st["learning_rate"]
            cache = nrc.NeuralRadianceCache()
            cache.initialize(config=net)
            self.caches.append(cache)

    def nrc_step(self, spp: int, train_iterations: int | None = None, new_sequence: bool = False) -> None:
        """One radiance-cache frame of every scene (its own cache's training iterations, then `spp`
        samples per pixel), each scene on its own stream forked from and joined to the caller's.
        Not captured in a graph: each frame draws the unbiased-path offsets on the host
        (renderer_main.cpp:1566)."""
        import torch

        iters = self.nrc_settings.get("train_iterations", 1) if train_iterations is None else train_iterations
        origin = torch.cuda.current_stream()
        for r, s, cache in zip(self.renderers, self.streams, self.caches):
            s.wait_stream(origin)
            r.nrc_frame(cache, iters, spp, new_sequence, s.cuda_stream)
        for s in self.streams:
            origin.wait_stream(s)

    def nrc_errors(self) -> int:
        return sum(r.device_errors() | c.device_errors() for r, c in zip(self.renderers, self.caches))

    def images(self) -> list[np.ndarray]:
        return [r.image() for r in self.renderers]

    def reset(self) -> None:
        for r in self.renderers:
            r.reset_accumulation()
