"""b2World_StepBatch: many independent worlds stepped together (phases on a host thread
pool with one batched flush per wait, or every world on its own stream) must end exactly
where stepping each world alone ends, and match the oracle."""
from __future__ import annotations

import ctypes
import os

import pytest

import box2d_gb300 as B
from conftest import lockstep

pytestmark = pytest.mark.gpu


def _scenes(lib, seeds):
    return [B.Scene(lib, B.BATCH_WORLD, 0, 0, 0, s, B.NO_CONTINUOUS) for s in seeds]


@pytest.mark.parametrize("threads", [1, 8])
def test_batch_step_equals_single_steps(gpu_lib, threads):
    seeds = list(range(101, 133))
    batch = _scenes(gpu_lib, seeds)
    single = _scenes(gpu_lib, seeds)
    try:
        handles = (ctypes.c_int * len(batch))(*[s.handle for s in batch])
        for _ in range(3):
            gpu_lib.b2s_step_batch(handles, len(batch), 1.0 / 60.0, 4, 20, threads)
            for s in single:
                s.step(20)
            for b, s in zip(batch, single):
                assert b.state_hash() == s.state_hash()
                assert (b.contacts() == s.contacts()).all()
    finally:
        for s in batch + single:
            s.close()


def test_move_events_of_a_batch(gpu_lib):
    """The move events read for a whole batch are each world's events in turn."""
    import numpy as np

    batch = _scenes(gpu_lib, list(range(301, 309)))
    try:
        handles = (ctypes.c_int * len(batch))(*[s.handle for s in batch])
        gpu_lib.b2s_step_batch(handles, len(batch), 1.0 / 60.0, 4, 5, 4)
        cap = sum(s.body_count for s in batch)
        many = np.zeros((cap, 4), np.float32)
        n = gpu_lib.b2s_move_events_many(handles, len(batch), many.ctypes.data, cap)
        each = np.concatenate([s.move_events().copy() for s in batch])
        assert n == len(each) > 0
        assert (many[:n] == each).all()
    finally:
        for s in batch:
            s.close()


def test_batch_worlds_match_oracle(gpu_lib, oracle):
    for seed in (12345, 12346):
        lockstep(gpu_lib, oracle, B.BATCH_WORLD, 0, 0, 0, seed, B.NO_CONTINUOUS, 120)


@pytest.mark.parametrize("mode", ["lockstep", "streams"])
@pytest.mark.parametrize("flags", [0, B.NO_CONTINUOUS])
def test_mixed_batch_equals_single_steps(gpu_lib, mode, flags):
    """Worlds of different kinds in one batch: small worlds (solved one CTA each in the
    batched flush), a jointed world, and a pyramid too heavy for one CTA (solved on its own
    stream in the last phase)."""
    specs = [(B.BATCH_WORLD, 0, 0, 0, s) for s in range(201, 213)]
    specs += [(B.JOINT_ZOO, 4, 0, 0, 3), (B.JOINT_MIX, 3, 0, 0, 6), (B.SHAPE_ZOO, 60, 0, 0, 4),
              (B.LARGE_PYRAMID, 40, 0, 0, 0)]
    batch = [B.Scene(gpu_lib, k, a, b, c, seed, flags) for k, a, b, c, seed in specs]
    single = [B.Scene(gpu_lib, k, a, b, c, seed, flags) for k, a, b, c, seed in specs]
    old = os.environ.get("B2G_BATCH")
    os.environ["B2G_BATCH"] = mode
    try:
        handles = (ctypes.c_int * len(batch))(*[s.handle for s in batch])
        for _ in range(4):
            gpu_lib.b2s_step_batch(handles, len(batch), 1.0 / 60.0, 4, 15, 8)
            for s in single:
                s.step(15)
            for b, s in zip(batch, single):
                assert b.state_hash() == s.state_hash()
                assert (b.contacts() == s.contacts()).all()
    finally:
        if old is None:
            os.environ.pop("B2G_BATCH", None)
        else:
            os.environ["B2G_BATCH"] = old
        for s in batch + single:
            s.close()
