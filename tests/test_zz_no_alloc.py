"""b2p_contacts_noalloc (the contact table built in a fixed device scratch array, no
allocation) must return exactly what b2p_contacts returns, on consecutive calls and
across steps, and refuse worlds larger than its scratch. Named to run after every other
test file, so it also covers a process whose device has already run everything else."""
from __future__ import annotations

import numpy as np
import pytest

import box2d_gb300 as B

pytestmark = pytest.mark.gpu

MAX_CONTACT_IDS = 32768


def _noalloc_table(lib, world_id: int, capacity: int) -> tuple[int, np.ndarray]:
    out = np.full((capacity, 8), -7, np.int32)
    n = lib.b2p_contacts_noalloc(world_id, out.ctypes.data, capacity)
    return n, out


@pytest.mark.parametrize("kind,a,b,c,seed,flags", [
    (B.LARGE_PYRAMID, 20, 0, 0, 0, 0),
    (B.SHAPE_ZOO, 150, 0, 0, 3, B.NO_CONTINUOUS),
    (B.JOINT_ZOO, 4, 0, 0, 2, B.NO_CONTINUOUS),
])
def test_noalloc_contact_table_matches_b2p_contacts(gpu_lib, kind, a, b, c, seed, flags):
    with B.Scene(gpu_lib, kind, a, b, c, seed, flags) as s:
        for step in range(3):
            s.step(20)
            expected = s.contacts()
            # two consecutive calls on the same state, then again after more steps
            for _ in range(2):
                n, table = _noalloc_table(gpu_lib, s.world_id, max(1, expected.shape[0]) + 4)
                assert n == expected.shape[0]
                assert (table[:n] == expected).all()
                assert (table[n:] == -7).all(), "rows past the count must stay untouched"


def test_noalloc_contact_table_in_a_sleeping_world(gpu_lib):
    """Islands fall asleep at the end of a step: their contacts leave the graph colors (the
    table reports color -1 for them) while the device color lists are refreshed only at
    the next step. A world woken between steps is refused until it is stepped again."""
    with B.Scene(gpu_lib, B.SLEEP_PYRAMIDS, 3, 8, 80) as s:
        saw_sleeping = False
        for _ in range(14):
            s.step(25)
            expected = s.contacts()
            n, table = _noalloc_table(gpu_lib, s.world_id, max(1, expected.shape[0]) + 4)
            assert n == expected.shape[0]
            assert (table[:n] == expected).all()
            saw_sleeping |= bool(((expected[:, 7] == 1) & (expected[:, 3] == -1)).any())
        assert saw_sleeping, "no touching contact of a sleeping island was seen"
        _, awake = s.awake()
        asleep = [i for i in range(1, len(awake)) if awake[i] == 0]
        assert asleep
        s.apply(["velocity", asleep[-1], 0.0, 3.0, 0.0])  # wakes that body's island between steps
        n, _ = _noalloc_table(gpu_lib, s.world_id, 16)
        assert n == -1
        s.step(1)
        expected = s.contacts()
        n, table = _noalloc_table(gpu_lib, s.world_id, max(1, expected.shape[0]))
        assert n == expected.shape[0] and (table[:n] == expected).all()


def test_noalloc_contact_table_small_capacity_reports_full_count(gpu_lib):
    with B.Scene(gpu_lib, B.LARGE_PYRAMID, 10, 0) as s:
        s.step(5)
        expected = s.contacts()
        assert expected.shape[0] > 8
        n, table = _noalloc_table(gpu_lib, s.world_id, 8)
        assert n == expected.shape[0]
        assert (table[:8] == expected[:8]).all()


def test_noalloc_contact_table_refuses_worlds_beyond_its_scratch(gpu_lib):
    # 20x20 pyramids hold more than 32768 contact ids after the first step
    with B.Scene(gpu_lib, B.MANY_PYRAMIDS_RAIN, 20, 10, 0, 0, B.NO_CONTINUOUS) as s:
        s.step(1)
        n, _ = _noalloc_table(gpu_lib, s.world_id, 16)
        assert n == -2
    # a never-stepped world is refused without touching the device
    with B.Scene(gpu_lib, B.LARGE_PYRAMID, 5, 0) as s:
        n, _ = _noalloc_table(gpu_lib, s.world_id, 16)
        assert n == -1
