"""The reference's default radiance-cache network (renderer_scene.cpp:50:
initialize(PositionEncoding::HashGrid, 2, 0.01f); network_interface.cu:50-122) on the GPU,
through the C ABI, against the oracle's restatement of the multiresolution hash encoding.

The hash grid is 16 levels x 2 features, at most 2^15 entries per level, base resolution 16,
per-level scale 2, followed by OneBlob(4) on the angles / roughness and identity on the
reflectances; 2 hidden layers of 64, output activation None, Adam (lr 1e-2, beta 0.9 / 0.99,
epsilon 1e-15, L2 1e-6 on the matrices) under an EMA (0.99). Tolerances as for the other
encodings: FP16 tables, weights and activations with FP32 accumulation against FP64 accumulation
with the same FP16 rounding points.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import orc
from rtc8_gb300 import nrc

from .test_gpu_nrc import _queries, _target

ROOT = Path(__file__).resolve().parents[1]

pytestmark = pytest.mark.gpu

HG = nrc.NRC_ENCODING_HASHGRID


def _cache(hidden=2, grid_scale=0.5, seed=0):
    """A hash-grid cache whose tables hold values of order `grid_scale` (the initial +-1e-4 would
    leave the encoded features near zero)."""
    cfg = nrc.default_config(HG)
    cfg.num_hidden_layers = hidden
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=cfg)
    w = cache.params()
    mlp = len(w) - orc.nrc_grid_params()
    rng = np.random.default_rng(seed)
    w[mlp:] = rng.uniform(-grid_scale, grid_scale, len(w) - mlp).astype(np.float32)
    cache.set_params(w)
    return cache, cfg, w, mlp


def test_reference_defaults_and_layout(cuda_device):
    cfg = nrc.default_config(HG)
    assert (cfg.num_hidden_layers, cfg.output_activation) == (2, nrc.NRC_OUTPUT_NONE)
    assert cfg.epsilon == pytest.approx(1e-15) and cfg.l2_reg == pytest.approx(1e-6)
    assert cfg.ema_decay == pytest.approx(0.99) and cfg.learning_rate == pytest.approx(1e-2)
    cache = nrc.NeuralRadianceCache()
    cache.initialize(nrc.PositionEncoding.HashGrid, 2, 1e-2)   # the reference's own call
    lay = cache.layout()
    # 16^3 entries at level 0, 32^3 = 2^15 at level 1, 2^15 (hashed) at levels 2..15
    assert orc.nrc_grid_params() == 2 * (4096 + 15 * 32768)
    assert lay["in"][0] == 64 and lay["L"] == 3
    assert lay["total"] == 64 * 64 + 64 * 64 + 64 * 16 + orc.nrc_grid_params()
    w = cache.params()
    mlp = len(w) - orc.nrc_grid_params()
    assert np.abs(w[mlp:]).max() <= 1e-4 and np.abs(w[mlp:]).max() > 0  # published initialisation
    cache.finalize()


def test_hashgrid_encoding_matches_oracle(cuda_device):
    import torch

    cache, cfg, w, mlp = _cache()
    n = 500
    q = _queries(n, 11, volume=False)
    q[:7, 0:3] = [[0, 0, 0], [1, 1, 1], [1, 0, 1], [0.5, 0.5, 0.5], [-0.1, 0.3, 1.2], [0.999, 0.001, 0.25],
                  [1 / 3, 2 / 3, 1 / 7]]          # corners, the clamp, exact lattice points
    out = torch.zeros((n, 64), dtype=torch.float32, device="cuda")
    cache.encode(None, torch.from_numpy(q).cuda(), n, out)
    torch.cuda.synchronize()
    ref = orc.nrc_encode(HG, q, w[mlp:]).astype(np.float16).astype(np.float32)
    got = out.cpu().numpy()
    np.testing.assert_allclose(got[:, :32], ref[:, :32], rtol=2e-3, atol=2e-3)
    np.testing.assert_allclose(got[:, 32:], ref[:, 32:], rtol=2e-3, atol=2e-3)
    assert np.abs(got[:, :32]).max() > 0.1
    cache.finalize()


def test_hashgrid_inference_matches_oracle(cuda_device):
    import torch

    cache, cfg, w, mlp = _cache()
    n = 1000
    q = _queries(n, 12, volume=False)
    out = torch.full((n, 3), -7.0, dtype=torch.float32, device="cuda")
    cache.infer(None, torch.from_numpy(q).cuda(), n, out)
    torch.cuda.synchronize()
    ref = orc.nrc_forward(HG, 2, cfg.output_activation, w, q)
    scale = np.abs(ref).max()
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=2e-2, atol=2e-2 * scale)
    assert cache.device_errors() == 0
    cache.finalize()


def test_hashgrid_gradients_loss_and_adam_match_oracle(cuda_device):
    """Loss and gradient of one batch (matrices and tables) against the FP64 oracle, then one Adam
    step: L2 on the matrices only, and table entries without gradient keep their value."""
    import torch

    cache, cfg, w0, mlp = _cache(grid_scale=0.3, seed=1)
    n = 640
    q = _queries(n, 13, volume=False)
    t = _target(q)
    loss = cache.train(None, torch.from_numpy(q).cuda(), torch.from_numpy(t).cuda(), n, loss=True)
    g_gpu = cache.gradients()
    ref_loss, g_ref = orc.nrc_loss_grad(HG, 2, cfg.output_activation, cfg.loss_scale, w0, q, t)
    assert loss == pytest.approx(ref_loss, rel=1e-3)
    for part in (slice(0, mlp), slice(mlp, None)):
        a, b = g_gpu[part], g_ref[part]
        rel = np.linalg.norm(a - b) / np.linalg.norm(b)
        cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b)))
        assert rel < 3e-2 and cos > 0.999, (part, rel, cos)
    touched = g_ref[mlp:] != 0
    assert 0 < touched.mean() < 0.5                          # a batch touches few hashed entries
    assert np.all(g_gpu[mlp:][~touched] == 0)                # and no other entry
    w1 = cache.params()
    lay = cache.layout()
    real = np.zeros(mlp, dtype=bool)
    off = 0
    for j, (fi, fo) in enumerate(zip(lay["in"], lay["out"])):
        m = np.zeros((fo, fi), bool)
        m[: (3 if j == lay["L"] - 1 else fo), : (58 if j == 0 else fi)] = True
        real[off: off + fo * fi] = m.reshape(-1)
        off += fo * fi
    assert off == mlp
    z = np.zeros(mlp, np.float32)
    ref_mlp, _, _ = orc.adam(w0[:mlp], z, z, g_gpu[:mlp], cfg.learning_rate, cfg.beta1, cfg.beta2, cfg.epsilon,
                             cfg.l2_reg, 1)
    np.testing.assert_allclose(w1[:mlp], np.where(real, ref_mlp, w0[:mlp]), rtol=1e-5, atol=1e-6)
    zg = np.zeros(len(w0) - mlp, np.float32)
    ref_grid, _, _ = orc.adam(w0[mlp:], zg, zg, g_gpu[mlp:], cfg.learning_rate, cfg.beta1, cfg.beta2, cfg.epsilon,
                              0.0, 1)
    sparse = g_gpu[mlp:] != 0
    np.testing.assert_allclose(w1[mlp:], np.where(sparse, ref_grid, w0[mlp:]), rtol=1e-5, atol=1e-6)
    cache.finalize()


def test_hashgrid_cache_fits_a_detailed_field(cuda_device):
    """Trained with the reference's settings on a radiance field with fine spatial detail, the
    hash-grid cache fits it far better than the TriangleWave cache of the same size does."""
    import torch

    def field(q):
        p = q[:, 0:3]
        base = 0.5 + 0.4 * np.sin(23 * p[:, 0:1] + 17 * p[:, 1:2]) * np.cos(19 * p[:, 2:3])
        return np.concatenate([base, 0.7 * base, 0.4 * base + 0.1], axis=1).astype(np.float32)

    losses = {}
    for enc in (nrc.PositionEncoding.HashGrid, nrc.PositionEncoding.TriangleWave):
        cache = nrc.NeuralRadianceCache()
        cache.initialize(enc, 2, 1e-2)
        n = 16384
        for step in range(400):
            q = _queries(n, 200 + step % 16, volume=False)
            cache.train(None, torch.from_numpy(q).cuda(), torch.from_numpy(field(q)).cuda(), n)
        q = _queries(n, 999, volume=False)
        out = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
        cache.infer(None, torch.from_numpy(q).cuda(), n, out)
        torch.cuda.synchronize()
        y, t = out.cpu().numpy(), field(q)
        losses[enc.name] = float(np.mean((y - t) ** 2) / np.mean(t ** 2))
        assert cache.device_errors() == 0
        cache.finalize()
    assert losses["HashGrid"] < 0.02, losses
    assert losses["HashGrid"] < 0.5 * losses["TriangleWave"], losses
