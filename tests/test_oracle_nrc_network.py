"""CPU checks of the oracle network itself (oracle/nrc_oracle.cpp), which the GPU MLP tests rely on:
the multiresolution hash encoding's lattice geometry and interpolation, and the analytic
gradient of the loss against central finite differences for matrices and hash-grid tables."""
import numpy as np
import pytest

from oracle import orc

HG = 2


def _queries(n, seed):
    rng = np.random.default_rng(seed)
    q = np.zeros((n, 14), np.float32)
    q[:, 0:3] = rng.random((n, 3))
    q[:, 3] = rng.random(n) * np.pi
    q[:, 4] = rng.random(n) * 2 * np.pi
    q[:, 5] = rng.random(n) * np.pi
    q[:, 6] = rng.random(n) * 2 * np.pi
    q[:, 7] = rng.random(n)
    q[:, 8:14] = rng.random((n, 6))
    return q


def _level_entry(level: int, x: int, y: int, z: int) -> int:
    """Entry index of lattice point (x, y, z) of one level (the published dense / hashed rule)."""
    res = 16 << level
    size = min(((res ** 3 + 7) // 8) * 8, 1 << 15)
    off = sum(min((((16 << l) ** 3 + 7) // 8) * 8, 1 << 15) for l in range(level))
    if res ** 3 <= size:
        i = x + (y + z * res) * res
    else:
        i = (x ^ ((y * 2654435761) & 0xFFFFFFFF) ^ ((z * 805459861) & 0xFFFFFFFF)) & 0xFFFFFFFF
    return off + i % size


def test_hash_grid_interpolates_lattice_values():
    """At a position that falls exactly on a lattice point of level l (x * scale + 1/2 with
    frac 0), the level's features are the entry of that point; halfway between two points along
    x they are the mean of the two."""
    G = orc.nrc_grid_params()
    assert G == 2 * (16 ** 3 + 15 * (1 << 15))
    rng = np.random.default_rng(0)
    grid = rng.uniform(-1, 1, G).astype(np.float16).astype(np.float32)
    # level 0: scale 15, lattice point k at x = (k - 0.5) / 15
    kx, ky, kz = 3, 7, 11
    q = np.zeros((2, 14), np.float32)
    q[0, 0:3] = [(kx - 0.5) / 15, (ky - 0.5) / 15, (kz - 0.5) / 15]
    q[1, 0:3] = [kx / 15, (ky - 0.5) / 15, (kz - 0.5) / 15]
    enc = orc.nrc_encode(HG, q, grid)
    e0 = _level_entry(0, kx, ky, kz)
    e1 = _level_entry(0, kx + 1, ky, kz)
    np.testing.assert_allclose(enc[0, 0:2], grid[2 * e0: 2 * e0 + 2], rtol=1e-6, atol=1e-7)
    np.testing.assert_allclose(enc[1, 0:2], 0.5 * (grid[2 * e0: 2 * e0 + 2] + grid[2 * e1: 2 * e1 + 2]),
                               rtol=1e-6, atol=1e-6)
    # a hashed level (level 5, scale 511) at a lattice point
    s5 = 16 * 32 - 1
    q[0, 0:3] = [(100 - 0.5) / s5, (200 - 0.5) / s5, (300 - 0.5) / s5]
    enc = orc.nrc_encode(HG, q[:1], grid)
    e = _level_entry(5, 100, 200, 300)
    np.testing.assert_allclose(enc[0, 10:12], grid[2 * e: 2 * e + 2], rtol=1e-4, atol=1e-5)
    # the rest of the input: OneBlob(4) on 5 values and identity on 6, then zeros
    assert enc.shape[1] == 64 and np.all(enc[:, 58:] == 0)


def test_hash_grid_gradient_matches_finite_differences():
    """The oracle's analytic loss gradient against central differences along random +-1
    directions over the hash-grid tables and over the matrices (loss scale 1). The relative L2
    loss holds its denominator (luminance^2 + 0.01 of the prediction) constant in the backward
    pass, so the differences are taken of the same loss with the denominator frozen at the
    unperturbed prediction, evaluated through the oracle's forward pass. That pass rounds the
    encoded input and the activations to FP16 like the GPU, so single coordinates are too coarse a
    probe; a direction over all touched parameters averages the rounding out."""
    rng = np.random.default_rng(3)
    hidden = 1
    G = orc.nrc_grid_params()
    mlp = int(orc.nrc_lib().orc_nrc_num_params(HG, hidden)) - G
    w = np.zeros(mlp + G, np.float32)
    w[:mlp] = rng.uniform(-0.3, 0.3, mlp)
    w[mlp:] = rng.uniform(-0.5, 0.5, G)
    w = w.astype(np.float16).astype(np.float32)
    n = 24
    q = _queries(n, 4)
    t = np.abs(rng.standard_normal((n, 3))).astype(np.float32)
    loss, g = orc.nrc_loss_grad(HG, hidden, 0, 1.0, w, q, t)
    y0 = orc.nrc_forward(HG, hidden, 0, w, q).astype(np.float64)
    lum = y0 @ np.array([0.2126, 0.7152, 0.0722])
    denom = lum * lum + 0.01

    def frozen_loss(params):
        y = orc.nrc_forward(HG, hidden, 0, params, q).astype(np.float64)
        return float(np.sum((y - t) ** 2 / denom[:, None]) / (3 * n))

    assert frozen_loss(w) == pytest.approx(loss, rel=1e-6)
    for part in (slice(mlp, None), slice(0, mlp)):
        d = np.zeros_like(w)
        idx = np.nonzero(g[part])[0] + part.start
        assert len(idx) > 0
        d[idx] = rng.choice([-1.0, 1.0], len(idx)).astype(np.float32)
        h = np.float32(2.0 ** -8)
        fd = (frozen_loss(w + h * d) - frozen_loss(w - h * d)) / (2 * h)
        analytic = float(g.astype(np.float64) @ d.astype(np.float64))
        assert fd == pytest.approx(analytic, rel=0.05), (part, fd, analytic)
