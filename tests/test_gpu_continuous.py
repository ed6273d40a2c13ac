"""Continuous collision on the GB300 path (solver.c:384-550 b2SolveContinuous): fast
non-bullet bodies swept against static shapes inside the finalize stage must land at the
oracle's time of impact, bit for bit, and the number of sweeps and hits must agree.
Tolerance: bit-exact (the library is built with --fmad=false, IEEE division and square
root)."""
from __future__ import annotations

import numpy as np
import pytest

import box2d_gb300 as B

pytestmark = pytest.mark.gpu

CONTINUOUS = 0


def _lockstep_continuous(gpu_lib, oracle, kind, a, b, c, seed, steps, check_every=1):
    with B.Scene(gpu_lib, kind, a, b, c, seed, CONTINUOUS) as g, B.Scene(oracle, kind, a, b, c, seed, CONTINUOUS) as o:
        for k in range(1, steps + 1):
            g.step()
            o.step()
            if k % check_every == 0 or k == steps:
                if g.state_hash() != o.state_hash():
                    gs, os_ = g.state(), o.state()
                    bad = np.nonzero((gs.view(np.uint32) != os_.view(np.uint32)).any(1))[0]
                    pytest.fail(f"state differs at step {k} in {len(bad)} bodies, first {bad[:5]}; "
                                f"sweeps/hits gpu {g.continuous_counts()} oracle {o.continuous_counts()}")
        gc, oc = g.contacts(), o.contacts()
        assert gc.shape == oc.shape and (gc == oc).all(), "contact tables differ"
        assert g.continuous_counts() == o.continuous_counts()
        return o.continuous_counts()


@pytest.mark.parametrize("seed", [1, 2, 3, 4])
def test_gpu_continuous_shape_zoo(gpu_lib, oracle, seed):
    """Circles, capsules, boxes and polygons thrown at a static segment and box floor."""
    sweeps, hits = _lockstep_continuous(gpu_lib, oracle, B.SHAPE_ZOO, 150, 0, 0, seed, 150)
    assert sweeps > 1000 and hits > 0


@pytest.mark.parametrize("seed", [21, 22, 23])
def test_gpu_continuous_batch_worlds(gpu_lib, oracle, seed):
    sweeps, hits = _lockstep_continuous(gpu_lib, oracle, B.BATCH_WORLD, 0, 0, 0, seed, 150)
    assert hits > 0


@pytest.mark.parametrize("seed", [5, 6, 7])
def test_gpu_continuous_joint_zoo(gpu_lib, oracle, seed):
    """Jointed mechanisms: the sweep skips static shapes joined to the fast body by a joint
    that does not collide its bodies (b2ShouldBodiesCollide)."""
    sweeps, hits = _lockstep_continuous(gpu_lib, oracle, B.JOINT_ZOO, 8, 0, 0, seed, 200)
    assert hits > 0


def test_gpu_continuous_rain(gpu_lib, oracle):
    """Rain of fast circles over a 3 x 3 field of pyramids: many sweeps, no static hit."""
    sweeps, hits = _lockstep_continuous(gpu_lib, oracle, B.MANY_PYRAMIDS_RAIN, 3, 3, 200, 0, 150, check_every=5)
    assert sweeps > 10000


def test_gpu_continuous_full_many_pyramids(gpu_lib, oracle):
    """Full-size many-pyramids-with-rain scene with continuous collision, 40 steps."""
    _lockstep_continuous(gpu_lib, oracle, B.MANY_PYRAMIDS_RAIN, 20, 10, 2000, 0, 40, check_every=10)


def test_gpu_continuous_joint_grid_mixed(gpu_lib, oracle):
    """Revolute circle grid with mixed shapes dropped on it, continuous collision on."""
    _lockstep_continuous(gpu_lib, oracle, B.JOINT_GRID_MIXED, 30, 200, 0, 9, 120, check_every=5)
