"""The three solver strategies of the GB300 library -- connected components in shared
memory (default), one launch per color stage, one cooperative launch -- must each match
the oracle bit for bit. The scenes cover worlds whose components are all small, worlds
that mix one big component with small ones, joints inside shared-memory bins, and
restitution."""
from __future__ import annotations

import pytest

import box2d_gb300 as B
from conftest import lockstep

pytestmark = pytest.mark.gpu

MODES = ["components", "launches", "persistent"]

# (id, kind, a, b, c, seed, flags, steps)
CASES = [
    ("pyramids_all_small", B.MANY_PYRAMIDS_RAIN, 4, 10, 200, 0, B.NO_CONTINUOUS, 60),
    ("pyramids_big_and_small", B.MANY_PYRAMIDS_RAIN, 2, 30, 600, 0, B.NO_CONTINUOUS, 40),
    ("joint_grid_in_bins", B.JOINT_GRID_MIXED, 6, 20, 0, 5, B.NO_CONTINUOUS, 80),
    ("joint_grid_big", B.JOINT_GRID_MIXED, 20, 60, 0, 5, B.NO_CONTINUOUS, 60),
    ("shape_zoo_restitution", B.SHAPE_ZOO, 150, 0, 0, 2, B.NO_CONTINUOUS, 100),
    ("batch_world", B.BATCH_WORLD, 0, 0, 0, 22, B.NO_CONTINUOUS, 100),
    ("joint_zoo", B.JOINT_ZOO, 6, 0, 0, 4, B.NO_CONTINUOUS, 150),
    ("joint_mix", B.JOINT_MIX, 6, 0, 0, 4, B.NO_CONTINUOUS, 150),
]


@pytest.mark.parametrize("mode", MODES)
@pytest.mark.parametrize("case", CASES, ids=[c[0] for c in CASES])
def test_solver_mode_matches_oracle(gpu_lib, oracle, monkeypatch, mode, case):
    monkeypatch.setenv("B2G_SOLVER", mode)
    _, kind, a, b, c, seed, flags, steps = case
    lockstep(gpu_lib, oracle, kind, a, b, c, seed, flags, steps)


# The cluster solver of the big components runs the warm start per body (fused with
# integrate velocities) when the cluster has no joints; B2G_CLUSTER_BODY_WARM=0 keeps the
# per-color warm start. Both must match the oracle bit for bit.
WARM_CASES = [
    ("pyramids_big_and_small", B.MANY_PYRAMIDS_RAIN, 2, 30, 600, 0, B.NO_CONTINUOUS, 40),
    ("pyramids_big_no_warm_start", B.MANY_PYRAMIDS_RAIN, 2, 30, 600, 0, B.NO_CONTINUOUS | B.NO_WARM_STARTING, 30),
    ("large_pyramid", B.LARGE_PYRAMID, 40, 1, 0, 0, 0, 40),
    ("shape_zoo_restitution", B.SHAPE_ZOO, 150, 0, 0, 2, B.NO_CONTINUOUS, 100),
]


@pytest.mark.parametrize("body_warm", ["1", "0"])
@pytest.mark.parametrize("case", WARM_CASES, ids=[c[0] for c in WARM_CASES])
def test_cluster_warm_start_per_body_matches_oracle(gpu_lib, oracle, monkeypatch, body_warm, case):
    monkeypatch.setenv("B2G_SOLVER", "components")
    monkeypatch.setenv("B2G_CLUSTER_BODY_WARM", body_warm)
    _, kind, a, b, c, seed, flags, steps = case
    lockstep(gpu_lib, oracle, kind, a, b, c, seed, flags, steps)


# Plain revolute joints (no spring, motor or limit) kept in a cluster CTA's shared memory read
# their constants from their slot; B2G_CLUSTER_JOINT_CONSTANTS=0 reads every joint's constant
# part from global memory. Both must match the oracle bit for bit.
JOINT_CONSTANT_CASES = [
    ("joint_grid_big", B.JOINT_GRID_MIXED, 20, 60, 0, 5, B.NO_CONTINUOUS, 60),
    ("joint_grid_no_warm_start", B.JOINT_GRID_MIXED, 20, 60, 0, 5, B.NO_CONTINUOUS | B.NO_WARM_STARTING, 30),
    ("joint_zoo", B.JOINT_ZOO, 6, 0, 0, 4, B.NO_CONTINUOUS, 150),
]


@pytest.mark.parametrize("constants", ["1", "0"])
@pytest.mark.parametrize("case", JOINT_CONSTANT_CASES, ids=[c[0] for c in JOINT_CONSTANT_CASES])
def test_cluster_joint_constants_match_oracle(gpu_lib, oracle, monkeypatch, constants, case):
    monkeypatch.setenv("B2G_SOLVER", "components")
    monkeypatch.setenv("B2G_CLUSTER_JOINT_CONSTANTS", constants)
    _, kind, a, b, c, seed, flags, steps = case
    lockstep(gpu_lib, oracle, kind, a, b, c, seed, flags, steps)
