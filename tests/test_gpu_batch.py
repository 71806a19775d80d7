"""Batched scenes (one CUDA graph per batch step) against the same launches issued one by one."""
import numpy as np
import pytest

from rtc8_gb300.batch import SceneBatch, make_c4_scenes
from rtc8_gb300.configs import VolumeSpec

from ._scenes import small_config_mode


def _configs():
    a = small_config_mode(size=48, n=32, g=0.4)
    b = small_config_mode(size=64, n=40, g=0.8).replace(volume=VolumeSpec(n=40, seed=7, octaves=4, threshold=0.4,
                                                                           sigma_t_max=30.0))
    c = small_config_mode(size=32, n=24, g=0.6).replace(rng_seed=12345)
    return [a, b, c]


@pytest.mark.gpu
def test_graph_replays_match_launches_issued_one_by_one(cuda_device):
    import torch

    spp = 2
    g = SceneBatch(_configs())
    g.capture(spp)
    g.step()
    g.step()
    torch.cuda.synchronize()
    got = [r.download_sum() for r in g.renderers]
    ref = SceneBatch(_configs())
    ref.step_uncaptured(spp)  # warm-up of capture() is one uncaptured step that is then reset
    torch.cuda.synchronize()
    ref.reset()
    ref.step_uncaptured(spp)
    ref.step_uncaptured(spp)
    torch.cuda.synchronize()
    for (sg, ng), r in zip(got, ref.renderers):
        sr, nr = r.download_sum()
        assert ng == nr == 2 * spp
        # FP64 sums of float samples added by atomics: equal up to the order of the additions
        np.testing.assert_allclose(sg, sr, rtol=1e-9, atol=1e-12)
        assert sg.max() > 0
    # a replay renders new samples: the second step changed every scene's image
    g.step()
    torch.cuda.synchronize()
    for (sg, _), r in zip(got, g.renderers):
        s3, n3 = r.download_sum()
        assert n3 == 3 * spp and not np.allclose(s3, sg)
    assert all(r.device_errors() == 0 for r in g.renderers)
    g.close()
    ref.close()


@pytest.mark.gpu
def test_autotuner_picks_a_shape_per_scene(cuda_device):
    g = SceneBatch(_configs()[:2])
    rep = g.autotune(spp=1, candidates=[(0, 0), (4, 16)])
    assert len(rep) == 2 and all(e["ms_per_launch"] > 0 for e in rep)
    assert all(r.download_sum()[1] == 0 for r in g.renderers)
    g.close()


def test_c4_scene_draw_is_seeded():
    a, b = make_c4_scenes(16, 4), make_c4_scenes(16, 4)
    assert [c.name for c in a] == [c.name for c in b]
    assert {c.width for c in a} <= {256, 512, 768, 1024}
    assert {c.volume.n for c in a} <= {64, 128, 256, 512}
    assert all(0.3 <= c.phase_param <= 0.9 for c in a)
