"""Scene generation is deterministic and describes the named workloads."""
import numpy as np

from box2dpp_gb300 import scenes


def test_splitmix_reference_values():
    r = scenes.SplitMix64(0)
    # splitmix64 published test vector for seed 0
    assert r.next_u64() == 0xE220A8397B1DCDAF


def test_pyramid_layout():
    s = scenes.config1()
    a = s.arrays()
    assert s.dynamic_count == 210 and len(a["body_type"]) == 211
    ys = a["body_f"][1:, 1]
    assert ys.min() == 0.5 and ys.max() == 19.5


def test_drop_deterministic_and_nonoverlapping():
    a1 = scenes.drop(400, scenes.SplitMix64(4)).arrays()
    a2 = scenes.drop(400, scenes.SplitMix64(4)).arrays()
    for k in a1:
        assert np.array_equal(a1[k], a2[k])
    pos = a1["body_f"][1:, :2]
    d = np.sqrt(((pos[:, None, :] - pos[None, :, :]) ** 2).sum(-1)) + np.eye(len(pos)) * 10
    assert d.min() > 0.5


def test_batched_counts_log_uniform():
    ws = scenes.config3(64, seed=3)
    n = np.array([w.dynamic_count for w in ws])
    assert n.min() >= 1 and n.max() <= 512
    kinds = {w.name.rstrip("0123456789") for w in ws}
    assert kinds == {"pyramid", "stacks", "drop"}
