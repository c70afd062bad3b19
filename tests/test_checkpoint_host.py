"""World checkpoints on the host (before any step, no GPU needed): a checkpoint restored into another
handle's world writes back the same bytes, keeps the broadphase tree, and malformed or foreign data
is refused without changing the world."""
from __future__ import annotations

import ctypes as C
import struct

import numpy as np
import pytest

from box2dpp_gb300 import scenes
from box2dpp_gb300._lib import GbError, WorldDef
from box2dpp_gb300.world import World
from tests._util import apply_ops, destroy_script


def _world():
    w = World(scenes.destroy_mix(scenes.SplitMix64(5)), track_tree=True)
    for _, ops in sorted(destroy_script().items())[:4]:
        apply_ops(w, ops)
    return w


def test_round_trip_into_another_handle():
    w = _world()
    data = w.checkpoint()
    v = World([scenes.pyramid(3), scenes.pyramid(4)], track_tree=True)
    v.restore(data, 1)
    assert v.checkpoint(1) == data
    assert v.tree_stats(1) == w.tree_stats()
    assert v.n_bodies[1] == w.n_bodies[0]
    # the other world of the batch is untouched
    assert v.checkpoint(0) == World([scenes.pyramid(3)], track_tree=True).checkpoint(0)


def test_restore_without_tree_tracking_target():
    data = _world().checkpoint()
    v = World([scenes.pyramid(3)])
    v.restore(data, 0)
    with pytest.raises(GbError):
        v.tree_stats(0)  # the handle does not track trees


@pytest.mark.parametrize("cut", [0, 4, 8, 40, 200, -1])
def test_truncated_checkpoints_are_refused(cut):
    data = _world().checkpoint()
    v = World([scenes.pyramid(3)])
    before = v.checkpoint(0)
    with pytest.raises(GbError):
        v.restore(data[:cut] if cut >= 0 else data[:-1], 0)
    assert v.checkpoint(0) == before


def test_foreign_and_corrupt_checkpoints_are_refused():
    src = _world()
    data = bytearray(src.checkpoint())
    v = World([scenes.pyramid(3)])
    bad_magic = bytes(b ^ 0xFF if i == 0 else b for i, b in enumerate(data))
    bad_version = data[:4] + struct.pack("<I", 99) + data[8:]
    bad_layout = bytearray(data)
    bad_layout[16] ^= 0x01  # the first record size of the layout column
    for blob in (bad_magic, bytes(bad_version), bytes(bad_layout), b"", bytes(100)):
        with pytest.raises(GbError):
            v.restore(blob, 0)
    # a body list head outside the bodies: magic, version, the 7-entry layout column, the world
    # definition, then the flags (auto-clear, body list head, ...)
    at = 8 + 8 + 7 * 4 + C.sizeof(WorldDef) + 4
    assert struct.unpack_from("<i", data, at)[0] == src.n_bodies[0] - 1  # the newest body heads the list
    bad_head = bytearray(data)
    struct.pack_into("<i", bad_head, at, 1_000_000)
    with pytest.raises(GbError):
        v.restore(bytes(bad_head), 0)
    with pytest.raises(GbError):
        v.restore(bytes(data) + b"\0", 0)  # trailing bytes


def test_corrupt_bytes_never_break_the_host():
    """Random byte corruption anywhere in a checkpoint: the restore is refused, or it is accepted only
    with every index the step follows in range, and the world can be checkpointed again."""
    import random

    w = World(scenes.destroy_mix(scenes.SplitMix64(5)))
    data = w.checkpoint()
    rng = random.Random(7)
    refused = accepted = 0
    for _ in range(300):
        blob = bytearray(data)
        for _ in range(rng.randint(1, 4)):
            blob[rng.randrange(len(blob))] = rng.randrange(256)
        v = World([scenes.pyramid(2)])
        try:
            v.restore(bytes(blob), 0)
        except GbError:
            refused += 1
            continue
        accepted += 1
        assert len(v.checkpoint(0)) == len(blob)
    assert refused > 0 and accepted > 0
