"""Parity at the benchmark workloads' own sizes and timed windows: the GB300 library must
match the oracle bit for bit (body states, contact tables) through the steps the bench
times, with the workloads' own flags (continuous collision on). The bench's default
window of the many-pyramids workload is steps 206-225, after the rain has reached the
pyramids; the joint grid and the batched worlds are checked at full size as well."""
from __future__ import annotations

import ctypes
import os

import numpy as np
import pytest

import box2d_gb300 as B

pytestmark = pytest.mark.gpu


@pytest.fixture()
def threaded_oracle(oracle):
    oracle.b2o_set_threads.argtypes = [ctypes.c_int]
    oracle.b2o_set_threads(max(1, os.cpu_count() or 1))
    yield oracle
    oracle.b2o_set_threads(1)


def _compare(g, o, k):
    if g.state_hash() != o.state_hash():
        gs, os_ = g.state(), o.state()
        bad = np.nonzero((gs.view(np.uint32) != os_.view(np.uint32)).any(1))[0]
        pytest.fail(f"state differs at step {k} in {len(bad)} bodies, first {bad[:5]}")


def _lockstep_window(gpu_lib, oracle, kind, a, b, c, seed, flags, steps, check_every):
    with B.Scene(gpu_lib, kind, a, b, c, seed, flags) as g, B.Scene(oracle, kind, a, b, c, seed, flags) as o:
        for k in range(1, steps + 1):
            g.step()
            o.step()
            if k % check_every == 0 or k == steps:
                _compare(g, o, k)
                gc, oc = g.contacts(), o.contacts()
                assert gc.shape == oc.shape and (gc == oc).all(), f"contact tables differ at step {k}"
        return g.dynamic_count, g.contacts(), g.continuous_counts()


def test_many_pyramids_through_the_timed_window(gpu_lib, threaded_oracle):
    """22000 boxes + 2000 rain circles, continuous collision on, steps 1-225 (the bench
    times 206-225 by default), checked every 25 steps."""
    dyn, table, (sweeps, hits) = _lockstep_window(gpu_lib, threaded_oracle, B.MANY_PYRAMIDS_RAIN, 20, 10, 2000, 0, 0,
                                                   225, 25)
    assert dyn == 24000
    assert table[:, 7].sum() > 60000  # the rain is on the pyramids: many touching contacts
    assert sweeps > 0


def test_joint_grid_full_size(gpu_lib, threaded_oracle):
    """100 x 100 revolute circle grid (19800 joints) + 3000 mixed shapes, continuous on,
    100 steps, checked every 20."""
    dyn, table, _ = _lockstep_window(gpu_lib, threaded_oracle, B.JOINT_GRID_MIXED, 100, 3000, 0, 0, 0, 100, 20)
    assert dyn > 12000 and table.shape[0] > 0


def test_large_pyramid_full_size_timed_window(gpu_lib, threaded_oracle):
    """5050-box pyramid, continuous on, steps 1-125 (the bench's window at --steps 100 is
    6-105), checked every 25 steps."""
    dyn, table, _ = _lockstep_window(gpu_lib, threaded_oracle, B.LARGE_PYRAMID, 100, 1, 0, 0, 0, 125, 25)
    assert dyn == 5050 and table[:, 7].sum() > 14000


def test_batched_worlds_of_the_batch_workload(gpu_lib, oracle):
    """64 worlds of the batched workload (seeds 12345 + index, continuous on) advanced by
    b2World_StepBatch for 300 steps must equal the oracle stepping each world alone."""
    n, steps = 64, 300
    gpu = [B.Scene(gpu_lib, B.BATCH_WORLD, 0, 0, 0, 12345 + i, 0) for i in range(n)]
    cpu = [B.Scene(oracle, B.BATCH_WORLD, 0, 0, 0, 12345 + i, 0) for i in range(n)]
    try:
        handles = (ctypes.c_int * n)(*[s.handle for s in gpu])
        for k in range(50, steps + 1, 50):
            gpu_lib.b2s_step_batch(handles, n, 1.0 / 60.0, 4, 50, 16)
            for s in cpu:
                s.step(50)
            for i, (g, o) in enumerate(zip(gpu, cpu)):
                assert g.state_hash() == o.state_hash(), f"world {i} differs at step {k}"
        for i, (g, o) in enumerate(zip(gpu, cpu)):
            assert (g.contacts() == o.contacts()).all(), f"world {i}: contact tables differ"
    finally:
        for s in gpu + cpu:
            s.close()


def test_overflow_color_is_exercised(gpu_lib):
    """The overflow scene puts contacts and joints past the graph's colors: color 23 (the
    overflow) holds contacts every step, so the overflow solver path runs; its parity is
    checked against the reference fixture overflow_2 in test_gpu_parity.py."""
    with B.Scene(gpu_lib, B.OVERFLOW, 2, 0, 0, 4, 0) as s:
        for _ in range(3):
            s.step(20)
            table = s.contacts()
            assert (table[:, 3] == 23).sum() >= 40
