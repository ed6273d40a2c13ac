"""Islands and sleeping on the GB300 library (island.c, solver_set.c and the sleep pass of
solver.c in the reference).

The reference's own determinism test (test/test_determinism.c) is the pin: the falling
hinges must fall asleep at step 274 with the transform hash 0xE86690F4. The sleeping
fixtures of tests/golden (recorded from the reference) are also checked per step, body
state and awake count, by test_gpu_parity.py; here the same scenes run through batched
stepping, where the sleep and wake work is recorded and replayed with the other worlds'."""
from __future__ import annotations

import ctypes

import numpy as np
import pytest

import box2d_gb300 as B
from conftest import load_golden

pytestmark = pytest.mark.gpu

# test/test_determinism.c:21-22 (float build)
EXPECTED_SLEEP_STEP = 274
EXPECTED_HASH = 0xE86690F4


def test_falling_hinges_determinism(gpu_lib):
    with B.Scene(gpu_lib, B.FALLING_HINGES, 0, 0, 0, 0, 0) as s:
        sleep_step, digest = s.run_until_asleep(500)
        assert (sleep_step, digest) == (EXPECTED_SLEEP_STEP, EXPECTED_HASH), (sleep_step, hex(digest))
        n, flags = s.awake()
        assert n == 0 and not flags.any()


def test_falling_hinges_repeatable(gpu_lib):
    """Three worlds at once give the same sleep step and hash (the test's multithreading
    loop, here several worlds sharing the device)."""
    scenes = [B.Scene(gpu_lib, B.FALLING_HINGES, 0, 0, 0, 0, 0) for _ in range(3)]
    try:
        results = [s.run_until_asleep(500) for s in scenes]
    finally:
        for s in scenes:
            s.close()
    assert results == [(EXPECTED_SLEEP_STEP, EXPECTED_HASH)] * 3


@pytest.mark.parametrize("name", ["sleep_pyramids_3x8", "sleep_api_pyramids", "falling_hinges"])
def test_sleeping_worlds_in_a_batch(gpu_lib, name):
    """Batched stepping of several copies of a sleeping scene matches the reference fixture
    step for step: islands fall asleep and wake inside the lockstep phases."""
    g = load_golden(name)
    script = g.get("script", [])
    scenes = [B.Scene(gpu_lib, g["kind"], g["a"], g["b"], g["c"], g["seed"], g["flags"]) for _ in range(3)]
    try:
        handles = (ctypes.c_int * len(scenes))(*[s.handle for s in scenes])
        for k, expected in enumerate(g["state_hashes"], start=1):
            gpu_lib.b2s_step_batch(handles, len(scenes), g["dt"], g["substeps"], 1, 4)
            for action in script:
                if action[0] == k:
                    for s in scenes:
                        s.apply(action[1:])
            for w, s in enumerate(scenes):
                assert f"{s.state_hash():016x}" == expected, f"{name}: world {w} differs at step {k}"
                assert s.awake()[0] == g["awake_counts"][k - 1], f"{name}: world {w} awake count at step {k}"
    finally:
        for s in scenes:
            s.close()


def test_move_events_report_falling_asleep(gpu_lib):
    """The step that puts islands to sleep still reports their bodies' moves, flagged as
    falling asleep; the next step reports none of them."""
    g = load_golden("falling_hinges")
    counts = g["awake_counts"]
    first = next(k for k in range(1, len(counts)) if counts[k] < counts[k - 1]) + 1  # 1-based step
    with B.Scene(gpu_lib, B.FALLING_HINGES, 0, 0, 0, 0, 0) as s:
        s.step(first - 1)
        n_before = s.awake()[0]
        s.step(1)
        buf = np.zeros(4 * 128, np.float32)
        moves = s.lib.b2s_move_events(s.handle, buf.ctypes.data, 128)
        assert moves == n_before
        assert s.awake()[0] == counts[first - 1] < n_before
        s.step(1)
        assert s.lib.b2s_move_events(s.handle, buf.ctypes.data, 128) == counts[first - 1]
