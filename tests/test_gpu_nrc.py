"""GPU radiance-cache MLP (tcgen05) against the oracle network, through the C ABI.

Tolerances: FP16 weights / activations with FP32 accumulation (GPU) against FP64 accumulation
with the same FP16 rounding points (oracle): outputs within 2e-2 relative, gradient vectors
within 3e-2 relative L2 error (cosine > 0.999), loss within 1e-3 relative, Adam updates within
1e-5 relative.
"""
from pathlib import Path

import numpy as np
import pytest

from oracle import orc
from rtc8_gb300 import nrc

ROOT = Path(__file__).resolve().parents[1]

pytestmark = pytest.mark.gpu


def _queries(n, seed=0, volume=True):
    rng = np.random.default_rng(seed)
    q = np.zeros((n, 14), np.float32)
    q[:, 0:3] = rng.random((n, 3))
    q[:, 3] = rng.random(n) * np.pi
    q[:, 4] = rng.random(n) * 2 * np.pi
    q[:, 5] = rng.random(n) * np.pi
    q[:, 6] = rng.random(n) * 2 * np.pi
    q[:, 7] = rng.random(n) if volume else 0.0
    q[:, 8:11] = rng.random((n, 3))
    q[:, 11:14] = 0.0 if volume else rng.random((n, 3))
    return q


def _target(q):
    """A smooth radiance-like field of position and direction."""
    p = q[:, 0:3]
    base = 0.5 + 0.4 * np.sin(3 * p[:, 0:1] + 2 * p[:, 1:2]) * np.cos(2 * p[:, 2:3] + q[:, 5:6])
    return np.concatenate([base, 0.8 * base, 0.6 * base + 0.1], axis=1).astype(np.float32)


@pytest.mark.parametrize("a_mode,b_mode", [(0, 0), (1, 1), (0, 1), (1, 0)])
def test_tensor_core_descriptor_layouts(cuda_device, a_mode, b_mode):
    rng = np.random.default_rng(a_mode * 2 + b_mode)
    a = rng.standard_normal((128, 64)).astype(np.float32)
    b = rng.standard_normal((64, 64)).astype(np.float32)
    ah = a.astype(np.float16).astype(np.float64)
    bh = b.astype(np.float16).astype(np.float64)
    ref = ah @ bh.T
    d = nrc.selftest_mma(a, b, a_mode, b_mode)
    err = np.abs(d - ref).max() / np.abs(ref).max()
    if err > 1e-3 and (a_mode or b_mode):
        alt = nrc.selftest_mma(a, b, 2 if a_mode else 0, 2 if b_mode else 0)
        alt_err = np.abs(alt - ref).max() / np.abs(ref).max()
        pytest.fail(f"MN-major layout mismatch: err {err:.3e}; exchanged offsets give {alt_err:.3e}")
    assert err < 1e-3


def test_mma_rate_probe(cuda_device):
    """The issue-rate probe behind the bench's MMA-shape ceiling: it completes, and wider MMAs
    take at least as long per instruction (an N = 256 MMA is four N = 64 MMAs of work)."""
    cyc = {n: nrc.selftest_mma_rate(n, 256) for n in (64, 256)}
    assert all(c > 0 for c in cyc.values())
    assert cyc[256] >= cyc[64]
    with pytest.raises(nrc.NrcError):
        nrc.selftest_mma_rate(72, 256)


@pytest.mark.parametrize("encoding", [nrc.NRC_ENCODING_REFERENCE, nrc.NRC_ENCODING_VOLUME])
def test_encodings_match_oracle(cuda_device, encoding):
    import torch

    cfg = nrc.default_config(encoding)
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=cfg)
    q = _queries(300, 1, volume=encoding == nrc.NRC_ENCODING_VOLUME)
    tq = torch.from_numpy(q).cuda()
    d = orc.nrc_lib().orc_nrc_in_dim(encoding)
    out = torch.zeros((300, d), dtype=torch.float32, device="cuda")
    cache.encode(None, tq, 300, out)
    torch.cuda.synchronize()
    ref = orc.nrc_encode(encoding, q).astype(np.float16).astype(np.float32)
    np.testing.assert_allclose(out.cpu().numpy(), ref, rtol=2e-3, atol=2e-3)
    cache.finalize()


@pytest.mark.parametrize("encoding,hidden", [(nrc.NRC_ENCODING_VOLUME, 5), (nrc.NRC_ENCODING_REFERENCE, 2)])
def test_inference_matches_oracle(cuda_device, encoding, hidden):
    import torch

    cfg = nrc.default_config(encoding)
    cfg.num_hidden_layers = hidden
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=cfg)
    w = cache.params()
    n = 1000  # not a multiple of 128
    q = _queries(n, 2, volume=encoding == nrc.NRC_ENCODING_VOLUME)
    tq = torch.from_numpy(q).cuda()
    out = torch.full((n, 3), -7.0, dtype=torch.float32, device="cuda")
    cache.infer(None, tq, n, out)
    torch.cuda.synchronize()
    ref = orc.nrc_forward(encoding, hidden, cfg.output_activation, w, q)
    got = out.cpu().numpy()
    scale = np.abs(ref).max()
    np.testing.assert_allclose(got, ref, rtol=2e-2, atol=2e-2 * scale)
    assert cache.device_errors() == 0
    cache.finalize()


def test_indexed_inference_matches_full_inference(cuda_device):
    """nrc_infer_indexed (the render pass lists the slots that hold a query): the listed records
    get exactly the full inference's values, in any list order, with the count read on the
    device; unlisted records keep their contents."""
    import torch

    cfg = nrc.default_config(nrc.NRC_ENCODING_VOLUME)
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=cfg)
    n = 5000
    q = torch.from_numpy(_queries(n, 4, volume=True)).cuda()
    full = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    cache.infer(None, q, n, full)
    rng = np.random.default_rng(9)
    listed = rng.permutation(n)[: 777].astype(np.uint32)  # not a multiple of 128, shuffled
    idx = torch.from_numpy(listed.view(np.int32)).cuda()
    count = torch.tensor([len(listed)], dtype=torch.int32, device="cuda")
    out = torch.full((n, 3), -5.0, dtype=torch.float32, device="cuda")
    cache.infer_indexed(None, q, idx, count, n, out)
    torch.cuda.synchronize()
    got, ref = out.cpu().numpy(), full.cpu().numpy()
    np.testing.assert_array_equal(got[listed], ref[listed])
    mask = np.ones(n, bool)
    mask[listed] = False
    assert np.all(got[mask] == -5.0)
    # an empty list leaves everything as it is
    count.zero_()
    out2 = torch.full((n, 3), 3.0, dtype=torch.float32, device="cuda")
    cache.infer_indexed(None, q, idx, count, n, out2)
    torch.cuda.synchronize()
    assert torch.all(out2 == 3.0)
    assert cache.device_errors() == 0
    cache.finalize()


@pytest.mark.parametrize("encoding,hidden", [(nrc.NRC_ENCODING_VOLUME, 5), (nrc.NRC_ENCODING_REFERENCE, 2)])
def test_gradients_loss_and_adam_match_oracle(cuda_device, encoding, hidden):
    import torch

    cfg = nrc.default_config(encoding)
    cfg.num_hidden_layers = hidden
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=cfg)
    w0 = cache.params()
    n = 640
    q = _queries(n, 3, volume=encoding == nrc.NRC_ENCODING_VOLUME)
    t = _target(q)
    loss = cache.train(None, torch.from_numpy(q).cuda(), torch.from_numpy(t).cuda(), n, loss=True)
    g_gpu = cache.gradients()
    ref_loss, g_ref = orc.nrc_loss_grad(encoding, hidden, cfg.output_activation, cfg.loss_scale, w0, q, t)
    assert loss == pytest.approx(ref_loss, rel=1e-3)
    rel = np.linalg.norm(g_gpu - g_ref) / np.linalg.norm(g_ref)
    cos = float(g_gpu @ g_ref / (np.linalg.norm(g_gpu) * np.linalg.norm(g_ref)))
    assert rel < 3e-2 and cos > 0.999, (rel, cos)
    # one Adam step on the GPU's own gradient, restated on the host
    w1 = cache.params()
    lay = cache.layout()
    ref_w1, _, _ = orc.adam(w0, np.zeros_like(w0), np.zeros_like(w0), g_gpu, cfg.learning_rate, cfg.beta1,
                            cfg.beta2, cfg.epsilon, cfg.l2_reg, 1)
    # padded rows / columns stay untouched; every real weight takes the Adam step (with L2)
    real = np.zeros_like(w0, dtype=bool)
    off = 0
    in_real = 138 if encoding == nrc.NRC_ENCODING_VOLUME else 62
    for j, (fi, fo) in enumerate(zip(lay["in"], lay["out"])):
        m = np.zeros((fo, fi), bool)
        m[: (3 if j == lay["L"] - 1 else fo), : (in_real if j == 0 else fi)] = True
        real[off: off + fo * fi] = m.reshape(-1)
        off += fo * fi
    assert off == lay["total"] == len(w0)
    np.testing.assert_allclose(w1, np.where(real, ref_w1, w0), rtol=1e-5, atol=1e-6)
    cache.finalize()


def test_training_reduces_loss(cuda_device):
    import torch

    cfg = nrc.default_config(nrc.NRC_ENCODING_VOLUME)
    cache = nrc.NeuralRadianceCache()
    cache.initialize(config=cfg)
    n = 16384
    rng = np.random.default_rng(5)
    losses = []
    for step in range(300):
        q = _queries(n, 100 + step % 8)
        t = _target(q)
        l = cache.train(None, torch.from_numpy(q).cuda(), torch.from_numpy(t).cuda(), n, loss=(step % 50 == 0 or step == 299))
        if l is not None:
            losses.append(l)
    assert losses[-1] < 0.2 * losses[0], losses
    assert cache.device_errors() == 0
    cache.finalize()


@pytest.mark.parametrize("encoding", ["TriangleWave", "HashGrid"])
def test_cpp_shim_matches_python_binding(cuda_device, tmp_path, encoding):
    """The reference's C++ interface (include/rtc8_nrc.hpp, rtc8::NeuralRadianceCache) used as the
    renderer uses it: initialize(<encoding>, 2, 1e-2) (renderer_scene.cpp:50 passes HashGrid), one
    train step with the loss read back, then inference, against the same calls through the Python
    binding (same default seed, so the same initial weights; gradients are reduced with atomics,
    hence the tolerance)."""
    import shutil
    import subprocess

    import torch

    from rtc8_gb300 import build

    cxx = shutil.which("g++")
    if cxx is None:
        pytest.skip("no C++ compiler")
    n = 512
    q = _queries(n, 7, volume=False)
    tgt = np.abs(np.random.default_rng(8).standard_normal((n, 3))).astype(np.float32)
    (tmp_path / "in.bin").write_bytes(q.astype(np.float32).tobytes() + tgt.tobytes())
    src = tmp_path / "shim.cpp"
    src.write_text(r'''
#include "rtc8_nrc.hpp"
#include <cuda_runtime.h>
#include <cstdio>
#include <vector>
int main(int argc, char** argv) {
    const unsigned n = 512;
    std::vector<float> h(n * 17), out(n * 3);
    FILE* f = std::fopen(argv[1], "rb");
    if (!f || std::fread(h.data(), sizeof(float), h.size(), f) != h.size()) return 2;
    std::fclose(f);
    float *d_in = nullptr, *d_tgt = nullptr, *d_out = nullptr;
    cudaMalloc(&d_in, n * 14 * sizeof(float));
    cudaMalloc(&d_tgt, n * 3 * sizeof(float));
    cudaMalloc(&d_out, n * 3 * sizeof(float));
    cudaMemcpy(d_in, h.data(), n * 14 * sizeof(float), cudaMemcpyHostToDevice);
    cudaMemcpy(d_tgt, h.data() + n * 14, n * 3 * sizeof(float), cudaMemcpyHostToDevice);
    rtc8::NeuralRadianceCache cache;
    cache.initialize(rtc8::PositionEncoding::ENCODING, 2, 1e-2f);
    float loss = 0.0f;
    cache.train(nullptr, d_in, d_tgt, n, &loss);
    cache.infer(nullptr, d_in, n, d_out);
    cudaMemcpy(out.data(), d_out, n * 3 * sizeof(float), cudaMemcpyDeviceToHost);
    f = std::fopen(argv[2], "wb");
    std::fwrite(&loss, sizeof(float), 1, f);
    std::fwrite(out.data(), sizeof(float), out.size(), f);
    std::fclose(f);
    cache.finalize();
    cudaFree(d_in); cudaFree(d_tgt); cudaFree(d_out);
    return 0;
}
''')
    libdir = build.LIB.parent
    cuda = Path(build.nvcc()).resolve().parent.parent
    exe = tmp_path / "shim"
    subprocess.run([cxx, "-std=c++17", f"-DENCODING={encoding}", "-I", str(ROOT / "include"), "-I",
                    str(cuda / "include"), str(src),
                    "-L", str(libdir), "-lrtc8_gb300", "-L", str(cuda / "lib64"), "-lcudart",
                    f"-Wl,-rpath,{libdir}", f"-Wl,-rpath,{cuda / 'lib64'}", "-o", str(exe)], check=True)
    subprocess.run([str(exe), str(tmp_path / "in.bin"), str(tmp_path / "out.bin")], check=True)
    res = np.frombuffer((tmp_path / "out.bin").read_bytes(), dtype=np.float32)
    loss_cpp, out_cpp = res[0], res[1:].reshape(n, 3)

    cache = nrc.NeuralRadianceCache()
    cache.initialize(nrc.PositionEncoding[encoding], 2, 1e-2)
    tq, tt = torch.from_numpy(q).cuda(), torch.from_numpy(tgt).cuda()
    loss_py = cache.train(None, tq, tt, n, loss=True)
    out = torch.zeros((n, 3), dtype=torch.float32, device="cuda")
    cache.infer(None, tq, n, out)
    torch.cuda.synchronize()
    assert loss_cpp == pytest.approx(loss_py, rel=1e-5)
    np.testing.assert_allclose(out_cpp, out.cpu().numpy(), rtol=1e-4, atol=1e-5)
    cache.finalize()
