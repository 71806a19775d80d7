"""The bench's reference arm (CPU, no GPU): one JSON line with the contract's keys, timed by the
host clock, the oracle's restatement on host-built inputs, and no GPU work."""
from __future__ import annotations

import json
from types import SimpleNamespace

import bench
from rtc8_gb300.configs import C1


def test_reference_arm_line():
    cfg = C1.replace(width=48, height=32)
    line = bench.reference_arm(SimpleNamespace(steps=1, warmup=0), cfg, 1)
    json.dumps(line)  # serialisable
    assert line["impl"] == "reference" and line["gpu_launches"] == 0
    for k in ("metric", "value", "unit", "n_gpus", "steps", "warmup", "ms_per_step", "higher_is_better", "scaling",
              "dtype", "data", "config", "cpu_baseline", "e2e"):
        assert k in line, k
    assert line["value"] > 0 and line["ms_per_step"] > 0
    assert abs(line["value"] - cfg.width * cfg.height * bench.STEP_SPP / (line["ms_per_step"] / 1e3)) < 1e-6 * line["value"]
    assert line["e2e"]["h2d_bytes_per_step"] == 0 and line["e2e"]["d2h_bytes_per_step"] == 0
    assert line["cpu_baseline"]["kind"] == "port" and line["cpu_baseline"]["cores"] >= 1
    assert line["config"]["workload"].startswith(cfg.name)
