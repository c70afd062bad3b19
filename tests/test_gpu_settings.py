"""b2World settings changed between device steps (SetGravity, SetAllowSleeping off and on,
SetWarmStarting, SetContinuousPhysics, SetSubStepping, SetAutoClearForces with a force kept across
steps, ClearForces): bit-exact against the reference's golden digests step by step, and the settings
of one world of a batch changed while the others step on."""
from __future__ import annotations

import numpy as np
import pytest

from box2dpp_gb300 import scenes
from box2dpp_gb300.world import World
from tests._util import DT, PI, VI, apply_ops, digest, golden, settings_script

pytestmark = pytest.mark.gpu


def test_settings_case_bit_exact_vs_reference(gpu):
    g = golden("settings_mix_project")
    w = World(scenes.destroy_mix(scenes.SplitMix64(7)))
    script = settings_script()
    for s in range(1, int(g["steps"]) + 1):
        if s in script:
            apply_ops(w, script[s])
        w.step(DT, VI, PI)
        assert np.array_equal(digest(w.bodies(), *w.contacts()), g["digests"][s - 1]), f"first divergence at step {s}"


def test_settings_in_one_world_of_a_batch(gpu):
    scs = [scenes.pyramid(6), scenes.destroy_mix(scenes.SplitMix64(7)), scenes.drop(120, scenes.SplitMix64(3))]
    alone = World([scs[0]])
    batch = World(scs)
    script = settings_script()
    for s in range(1, 201):
        if s in script:
            apply_ops(batch, script[s], w=1)
        batch.step(DT, VI, PI)
        alone.step(DT, VI, PI)
    batch.sync()
    alone.sync()
    # world 0 of the batch is untouched by world 1's settings
    assert np.array_equal(batch.bodies(0).view(np.uint32), alone.bodies(0).view(np.uint32))
