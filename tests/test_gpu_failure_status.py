"""Failure detection without a GPU fault: each device check reports through the world's
status word (b2p_status: the status bits of every step since the world was created), which
the host reads, and the device stays usable.

- a body given a non-finite velocity through b2Body_SetLinearVelocity: B2G_STATUS_NAN (1);
- the pair query's traversal stack made too small for the tree (B2G_PAIR_STACK_LIMIT):
  B2G_STATUS_CAPACITY (2);
- the persistent solver's grid barrier given almost no patience (B2G_PERSISTENT_SPIN_LIMIT):
  the barrier gives up, every block leaves, and the step reports the timeout (4).

The last two change process-wide settings, so they run in a child process."""
from __future__ import annotations

import math
import os
import subprocess
import sys
from pathlib import Path

import pytest

import box2d_gb300 as B

pytestmark = pytest.mark.gpu

ROOT = Path(__file__).resolve().parents[1]

STATUS_NAN, STATUS_CAPACITY, STATUS_PERSISTENT_TIMEOUT = 1, 2, 4

CHILD = r"""
import sys
sys.path.insert(0, {root!r})
import box2d_gb300 as B
lib = B.load_library()
with B.Scene(lib, B.LARGE_PYRAMID, {rows}, 0) as s:
    s.step({steps})
    print(lib.b2p_status(s.world_id))
# the device still works: a fresh world steps and reports no error
with B.Scene(lib, B.HELLO_WORLD) as s:
    s.step(5)
    print(lib.b2p_status(s.world_id))
"""


def _child(env_extra: dict, rows: int, steps: int) -> tuple[int, int]:
    env = dict(os.environ)
    env.update(env_extra)
    code = CHILD.format(root=str(ROOT), rows=rows, steps=steps)
    proc = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, env=env, timeout=300)
    assert proc.returncode == 0, proc.stderr
    lines = proc.stdout.split()
    return int(lines[-2]), int(lines[-1])


def test_non_finite_velocity_is_reported(gpu_lib):
    with B.Scene(gpu_lib, B.SHAPE_ZOO, 40, 0, 0, 3, 0) as s:
        s.step(2)
        assert gpu_lib.b2p_status(s.world_id) == 0
        s.apply(["velocity", 5, math.nan, 0.0, 0.0])
        s.step(1)
        assert gpu_lib.b2p_status(s.world_id) & STATUS_NAN


def test_exhausted_pair_stack_is_reported():
    status, fresh = _child({"B2G_PAIR_STACK_LIMIT": "2"}, rows=20, steps=2)
    assert status & STATUS_CAPACITY
    assert fresh & STATUS_NAN == 0  # the next world still steps (the small stack stays for the process)


def test_persistent_barrier_timeout_is_reported():
    status, fresh = _child({"B2G_SOLVER": "persistent", "B2G_PERSISTENT_SPIN_LIMIT": "1"}, rows=40, steps=1)
    assert status & STATUS_PERSISTENT_TIMEOUT
    assert fresh == 0  # a one-block grid never waits at a barrier: the device is usable
