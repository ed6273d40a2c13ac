"""World snapshots (b2World_Snapshot, b2World_Restore, b2CreateWorldFromSnapshot) on the GB300
library, in the manner of the reference's test/test_snapshot.c:
- a world created from a snapshot has the original's b2World_GetStateHash and steps in
  lockstep with it (state hash and body state every step);
- an in-place restore rolls the world back exactly: the state hash of the snapshot instant
  comes back, ids held from that instant stay valid, an id minted after it fails;
- a rejected image (none, a broken magic, a cut payload, a flipped payload byte) returns false
  and leaves the world unchanged; repeated restores give the same world;
- an image restores into another world, which then steps like a world created from it.

The fixtures snapshot_* (recorded from the reference, which restores through its own
snapshot code) check restores against the reference step by step in test_gpu_parity.py."""
from __future__ import annotations

import numpy as np
import pytest

import box2d_gb300 as B

pytestmark = pytest.mark.gpu


def _asleep_world(lib) -> B.Scene:
    s = B.Scene(lib, B.SLEEP_PYRAMIDS, 2, 6, 1000)
    s.step(95)
    assert s.awake()[0] < s.body_count  # sleeping solver sets exist
    return s


@pytest.mark.parametrize("kind,a,b,c,seed,flags,steps", [
    (B.SLEEP_PYRAMIDS, 2, 6, 1000, 0, 0, 95),
    (B.JOINT_ZOO, 4, 0, 0, 3, 0, 40),
    (B.SENSOR_ZOO, 60, 0, 0, 6, 0, 50),
    (B.CHAIN_ZOO, 80, 0, 0, 3, 0, 60),
    (B.MANY_PYRAMIDS_RAIN, 3, 10, 100, 0, 0, 120),
])
def test_world_from_snapshot_steps_in_lockstep(gpu_lib, kind, a, b, c, seed, flags, steps):
    with B.Scene(gpu_lib, kind, a, b, c, seed, flags) as s:
        s.step(steps)
        assert s.snapshot() > 0
        t = s.from_snapshot()
        try:
            assert t.world_state_hash() == s.world_state_hash()
            assert t.state_hash() == s.state_hash()
            for k in range(120):
                s.step()
                t.step()
                assert t.world_state_hash() == s.world_state_hash(), f"state hash differs {k + 1} steps after the snapshot"
                assert np.array_equal(t.state(), s.state()), f"body state differs {k + 1} steps after the snapshot"
        finally:
            t.close()


def test_restore_in_place_rolls_back_and_keeps_held_ids(gpu_lib):
    with _asleep_world(gpu_lib) as s:
        image = s.snapshot_image()
        snap_hash = s.world_state_hash()
        s.apply(["velocity", 3, 3.0, 6.0, 0.0])
        s.apply(["awake", 3, 1])
        late = s.add_box(20.0, 20.0)
        s.step(30)
        assert s.world_state_hash() != snap_hash
        assert s.restore_image(image)
        assert s.world_state_hash() == snap_hash
        assert all(s.body_valid(i) for i in range(late))
        assert not s.body_valid(late), "an id minted after the snapshot must fail validation"
        # the rolled-back world continues as a world created from the same image (the scene's
        # body list still names the late body, so only world-level hashes are compared)
        s.lib.b2s_snapshot(s.handle)
        t = s.from_snapshot()
        try:
            for k in range(60):
                s.step()
                t.step()
                assert s.world_state_hash() == t.world_state_hash(), k
        finally:
            t.close()


def test_rejected_images_leave_the_world_unchanged(gpu_lib):
    with _asleep_world(gpu_lib) as s:
        image = s.snapshot_image()
        s.step(10)
        before = s.world_state_hash()
        assert not s.restore_image(None)
        broken = bytearray(image)
        broken[0] ^= 0xFF  # the magic
        assert not s.restore_image(bytes(broken))
        assert not s.restore_image(image[:-16])  # cut short
        flipped = bytearray(image)
        flipped[len(image) // 2] ^= 0x01  # a payload byte: the checksum no longer matches
        assert not s.restore_image(bytes(flipped))
        assert s.world_state_hash() == before
        s.step(5)  # the world still steps
        for _ in range(3):
            assert s.restore_image(image)
        h = s.world_state_hash()
        s.step(20)
        assert s.restore_image(image)
        assert s.world_state_hash() == h


def test_image_restores_into_another_world(gpu_lib):
    with _asleep_world(gpu_lib) as s, B.Scene(gpu_lib, B.HELLO_WORLD) as other:
        image = s.snapshot_image()
        s.lib.b2s_snapshot(s.handle)
        fresh = s.from_snapshot()
        try:
            assert other.restore_image(image)
            wid = B.WorldId.unpack(other.world_id)
            assert gpu_lib.b2World_GetStateHash(wid) == fresh.world_state_hash()
            for k in range(120):
                other.step()
                fresh.step()
                assert gpu_lib.b2World_GetStateHash(wid) == fresh.world_state_hash(), k
        finally:
            fresh.close()


def test_snapshot_size_query_and_small_buffer(gpu_lib):
    import ctypes

    with B.Scene(gpu_lib, B.LARGE_PYRAMID, 10, 0) as s:
        s.step(3)
        wid = B.WorldId.unpack(s.world_id)
        size = gpu_lib.b2World_Snapshot(wid, None, 0)
        assert size > 0
        small = ctypes.create_string_buffer(b"\x5a" * 64, 64)
        assert gpu_lib.b2World_Snapshot(wid, small, 64) == size
        assert small.raw == b"\x5a" * 64, "nothing is written when the buffer is too small"
        assert len(s.snapshot_image()) == size
