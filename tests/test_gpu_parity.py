"""Parity of the GB300 library with the reference: per-step body-state hashes and
contact tables must match the golden fixtures recorded from the reference, and the live
CPU oracle on further seeds and at full benchmark sizes. Tolerance: bit-exact (the
library is built with --fmad=false, IEEE division and square root)."""
from __future__ import annotations

import hashlib

import numpy as np
import pytest

import box2d_gb300 as B
from conftest import EventCheck, golden_cases, load_golden, lockstep

pytestmark = pytest.mark.gpu


@pytest.mark.parametrize("name", golden_cases())
def test_gpu_matches_reference_fixture(gpu_lib, name):
    g = load_golden(name)
    with B.Scene(gpu_lib, g["kind"], g["a"], g["b"], g["c"], g["seed"], g["flags"]) as s:
        assert s.body_count == g["bodies"]
        script = g.get("script", [])
        events = EventCheck(g)
        sensor_events = EventCheck(g, "sensor_events")
        for k, expected in enumerate(g["state_hashes"], start=1):
            s.step(1, g["dt"], g["substeps"])
            events.step(s, k)
            sensor_events.step(s, k)
            for action in script:
                if action[0] == k:
                    s.apply(action[1:])
            assert f"{s.state_hash():016x}" == expected, f"{name}: body state differs from the reference at step {k}"
            if "world_state_hashes" in g:
                assert f"{s.world_state_hash():016x}" == g["world_state_hashes"][k - 1], \
                    f"{name}: b2World_GetStateHash (state and bookkeeping) differs from the reference at step {k}"
            if "awake_counts" in g:
                assert s.awake()[0] == g["awake_counts"][k - 1], f"{name}: awake body count at step {k}"
            d = g["contact_digests"].get(str(k))
            if d is not None:
                table = s.contacts()
                assert table.shape[0] == d["count"], f"{name}: contact count at step {k}"
                assert hashlib.sha256(table.astype("<i4").tobytes()).hexdigest() == d["sha256"], \
                    f"{name}: contact table (ids, pairs, colors, feature ids) at step {k}"
        events.finish(len(g["state_hashes"]))
        sensor_events.finish(len(g["state_hashes"]))


def _lockstep(*args, **kw):
    return lockstep(*args, **kw)


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_gpu_vs_oracle_shape_zoo_seeds(gpu_lib, oracle, seed):
    _lockstep(gpu_lib, oracle, B.SHAPE_ZOO, 150, 0, 0, seed, B.NO_CONTINUOUS, 150)


@pytest.mark.parametrize("seed", [21, 22, 23])
def test_gpu_vs_oracle_batch_worlds(gpu_lib, oracle, seed):
    _lockstep(gpu_lib, oracle, B.BATCH_WORLD, 0, 0, 0, seed, B.NO_CONTINUOUS, 150)


@pytest.mark.parametrize("seed", [5, 6, 7])
def test_gpu_vs_oracle_joint_zoo(gpu_lib, oracle, seed):
    """Prismatic, weld, wheel, distance and revolute joints with limits, motors and springs."""
    _lockstep(gpu_lib, oracle, B.JOINT_ZOO, 8, 0, 0, seed, B.NO_CONTINUOUS, 200)


@pytest.mark.parametrize("seed", [5, 6])
def test_gpu_vs_oracle_joint_mix(gpu_lib, oracle, seed):
    """Motor joints (velocity and spring control, between two dynamic bodies), pogo,
    mover and filter joints, with contacts on the motor-driven bodies."""
    _lockstep(gpu_lib, oracle, B.JOINT_MIX, 8, 0, 0, seed, B.NO_CONTINUOUS, 200)


def test_gpu_filter_joint_stops_collision(gpu_lib):
    """The two overlapping boxes joined by a filter joint never get a contact: the
    scene's contact table holds no pair of their shapes."""
    with B.Scene(gpu_lib, B.JOINT_MIX, 1, 0, 0, 5, B.NO_CONTINUOUS) as s:
        s.step(30)
        table = s.contacts()
    # cell 0: ground segment shape 0, motor box 1, ball 2, friction pair 3-4, pogo mover 5,
    # mover-walked box 6, filtered pair 7-8 (shape ids in creation order)
    pairs = {tuple(sorted((int(r[1]), int(r[2])))) for r in table}
    assert (7, 8) not in pairs
    assert any(7 in p or 8 in p for p in pairs)  # they still touch the ground


def test_gpu_vs_oracle_joint_grid_mixed(gpu_lib, oracle):
    _lockstep(gpu_lib, oracle, B.JOINT_GRID_MIXED, 30, 200, 0, 9, B.NO_CONTINUOUS, 120)


def test_gpu_vs_oracle_full_large_pyramid(gpu_lib, oracle):
    """Full-size large pyramid (5050 boxes, segment ground) for 100 steps."""
    bodies, contacts = _lockstep(gpu_lib, oracle, B.LARGE_PYRAMID, 100, 1, 0, 0, 0, 100, check_every=10)
    assert bodies == 5051 and contacts > 14000


def test_gpu_vs_oracle_full_many_pyramids(gpu_lib, oracle):
    """Full-size many-pyramids-with-rain scene (22000 boxes + 2000 circles), 40 steps."""
    bodies, contacts = _lockstep(gpu_lib, oracle, B.MANY_PYRAMIDS_RAIN, 20, 10, 2000, 0, B.NO_CONTINUOUS, 40,
                                 check_every=10)
    assert bodies == 24001


def test_gpu_edge_cases(gpu_lib, oracle):
    # a world whose only body is a dropped box (single contact life cycle), zero and
    # one substep, and a zero time step (collide only, no solve)
    for substeps in (1, 4):
        with B.Scene(gpu_lib, B.HELLO_WORLD) as g, B.Scene(oracle, B.HELLO_WORLD) as o:
            for k in range(40):
                g.step(1, 1.0 / 60.0, substeps)
                o.step(1, 1.0 / 60.0, substeps)
                assert g.state_hash() == o.state_hash(), (substeps, k)
    with B.Scene(gpu_lib, B.LARGE_PYRAMID, 5, 0) as g, B.Scene(oracle, B.LARGE_PYRAMID, 5, 0) as o:
        g.step(1, 0.0, 4)
        o.step(1, 0.0, 4)
        assert g.state_hash() == o.state_hash()
        assert (g.contacts() == o.contacts()).all()
        g.step(5)
        o.step(5)
        assert g.state_hash() == o.state_hash()


def test_gpu_empty_world(gpu_lib):
    with B.Scene(gpu_lib, B.LARGE_PYRAMID, 0, 0) as g:
        g.step(3)
        assert g.body_count == 1
        assert g.contacts().shape[0] == 0
