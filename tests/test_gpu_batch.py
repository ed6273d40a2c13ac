"""b2World_StepBatch: many independent worlds stepped together (host thread pool, one
stream per world) must end exactly where stepping each world alone ends, and match the
oracle."""
from __future__ import annotations

import ctypes

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


def test_batch_worlds_match_oracle(gpu_lib, oracle):
    for seed in (12345, 12346):
        lockstep(gpu_lib, oracle, B.BATCH_WORLD, 0, 0, 0, seed, B.NO_CONTINUOUS, 120)
