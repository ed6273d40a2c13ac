"""Adjoint of the recorded GB300 step (box2d_gb300_diff.h) on the differentiable-batch scene:
8 x 8 boxes of 0.5 m stacked on a static ramp, loss = squared distance of the final center
of mass to a seeded target. The gradient with respect to the initial velocities and the
shape frictions is checked against
  - the FP64 tangent-linear model of the same recorded steps (oracle/o_tangent.cpp):
    relative error of directional derivatives <= 1e-3;
  - central finite differences of the forward step: over 2 steps of the stacked boxes
    (h = 1e-3), <= 2e-2, where contacts switching under the perturbation make differences
    coarse; and for one box sliding on the ramp over 5 steps (h = 1e-2), a regime smooth
    enough for differences to resolve the derivative, <= 1e-3.

The tangent-linear checker is independent of the product: its dual numbers and its
polygon contact Jacobian are its own, restated from the reference. Rounded boxes with
rolling resistance check the rolling impulse's derivative the same way.
"""
from __future__ import annotations

import numpy as np
import pytest

import box2d_gb300 as B
from box2d_gb300.diff import DiffBatch

pytestmark = pytest.mark.gpu


def _make(lib, seeds, columns=8, rows=8, flags=0):
    batch = DiffBatch(lib, B.RAMP_WORLD, columns, rows, 0, seeds, flags)
    batch.dynamic_masks = [np.arange(s.body_count) > 0 for s in batch.scenes]  # body 0 is the ramp
    targets = np.zeros((len(seeds), 2))
    for w, s in enumerate(batch.scenes):
        t = np.zeros(2, np.float32)
        lib.b2s_target(s.handle, t.ctypes.data)
        targets[w] = t
    return batch, targets


def _loss_and_grad_centers(batch: DiffBatch, targets: np.ndarray):
    """L = sum over worlds of |mean dynamic center - target|^2, and dL/d(center)."""
    loss = 0.0
    grads = []
    for w, c in enumerate(batch.centers()):
        dyn = batch.dynamic_masks[w]
        d = c[dyn].astype(np.float64).mean(0) - targets[w]
        loss += float(d @ d)
        g = np.zeros_like(c)
        g[dyn] = (2.0 * d / dyn.sum()).astype(np.float32)
        grads.append(g)
    return loss, grads


def _run(batch, v0, f0, steps):
    batch.reset()
    batch.set_velocities(v0)
    batch.set_friction(f0)
    batch.step(steps)


def _direction(batch, v0, f0, rng):
    du = [rng.standard_normal(v.shape).astype(np.float32) * batch.dynamic_masks[w][:, None] for w, v in enumerate(v0)]
    df = [rng.standard_normal(f.shape).astype(np.float32) for f in f0]
    for f in df:
        f[0] = 0.0  # the ramp's friction stays fixed
    return du, df


def _tangent_derivative(tangent, batch, w, du, df, gc):
    """Directional derivative of the loss in world w from the FP64 tangent-linear model."""
    tape = np.frombuffer(batch.download_tape(w), np.uint8).copy()
    nb = int(batch.body_counts[w])
    dv = np.zeros((nb, 3), np.float32)
    dv[batch.body_ids[w]] = du[w]
    dc = np.zeros((nb, 2), np.float64)
    vel = np.zeros((nb, 3), np.float64)
    df_ = np.ascontiguousarray(df[w], np.float32)
    rc = tangent.b2t_tangent(tape.ctypes.data, tape.size, dv.ctypes.data, df_.ctypes.data, dc.ctypes.data, vel.ctypes.data)
    assert rc == 0, f"tangent-linear replay failed ({rc})"
    g = np.zeros((nb, 2), np.float64)
    g[batch.body_ids[w]] = gc[w]
    return float((g * dc).sum())


def test_adjoint_runs_on_the_ramp_batch(gpu_lib):
    batch, targets = _make(gpu_lib, [12345 + i for i in range(16)])
    with batch:
        v0, f0 = batch.velocities(), batch.friction()
        _run(batch, v0, f0, 60)
        assert batch.step_count() == 60
        loss, gc = _loss_and_grad_centers(batch, targets)
        gv, _, gf = batch.backward(gc)
        assert all(np.isfinite(g).all() for g in gv) and all(np.isfinite(g).all() for g in gf)
        assert any(np.abs(g).max() > 0 for g in gv)
        assert any(np.abs(g).max() > 0 for g in gf)
        ms, launches = batch.backward_ms()
        assert ms > 0 and launches == 62


@pytest.mark.parametrize("steps", [1, 5, 30, 120])
def test_adjoint_matches_tangent_linear(gpu_lib, tangent, steps):
    seeds = [901, 902, 903]
    batch, targets = _make(gpu_lib, seeds)
    rng = np.random.default_rng(steps)
    with batch:
        v0, f0 = batch.velocities(), batch.friction()
        _run(batch, v0, f0, steps)
        _, gc = _loss_and_grad_centers(batch, targets)
        gv, _, gf = batch.backward(gc)
        for trial in range(3):
            du, df = _direction(batch, v0, f0, rng)
            for w in range(len(seeds)):
                adjoint = float((gv[w].astype(np.float64) * du[w]).sum() + (gf[w].astype(np.float64) * df[w]).sum())
                tl = _tangent_derivative(tangent, batch, w, du, df, gc)
                assert abs(adjoint - tl) <= 1e-3 * max(abs(tl), 1e-6), (steps, w, trial, adjoint, tl)


@pytest.mark.parametrize("steps", [1, 10, 60])
def test_adjoint_with_rolling_resistance_matches_tangent_linear(gpu_lib, tangent, steps):
    """Rounded boxes with rolling resistance (contact_solver.c:2021-2031): the rolling
    impulse's clamp, its warm start and its carry between steps are differentiated."""
    seeds = [905, 906]
    batch, targets = _make(gpu_lib, seeds, flags=B.ROLLING_RESISTANCE)
    rng = np.random.default_rng(100 + steps)
    with batch:
        v0, f0 = batch.velocities(), batch.friction()
        _run(batch, v0, f0, steps)
        _, gc = _loss_and_grad_centers(batch, targets)
        gv, _, gf = batch.backward(gc)
        for trial in range(3):
            du, df = _direction(batch, v0, f0, rng)
            for w in range(len(seeds)):
                adjoint = float((gv[w].astype(np.float64) * du[w]).sum() + (gf[w].astype(np.float64) * df[w]).sum())
                tl = _tangent_derivative(tangent, batch, w, du, df, gc)
                assert abs(adjoint - tl) <= 1e-3 * max(abs(tl), 1e-6), (steps, w, trial, adjoint, tl)


@pytest.mark.parametrize("flags", [B.BALLS, B.BALLS | B.ROLLING_RESISTANCE, B.CAPSULES, B.SEGMENT_RAMP])
@pytest.mark.parametrize("steps", [1, 10, 60])
def test_adjoint_with_balls_matches_tangent_linear(gpu_lib, tangent, steps, flags):
    """Boxes with balls on the ramp: polygon-circle (manifold.c:127-230) and circle-circle
    (manifold.c:36-66) manifolds, with rolling resistance on the balls and rounded boxes
    in the second case; boxes with capsules (polygon-capsule, manifold.c:504-508), and boxes
    on a segment ramp (segment-polygon, manifold.c:1036-1040)."""
    seeds = [907, 908]
    batch, targets = _make(gpu_lib, seeds, flags=flags)
    rng = np.random.default_rng(200 + steps + flags)
    with batch:
        v0, f0 = batch.velocities(), batch.friction()
        _run(batch, v0, f0, steps)
        _, gc = _loss_and_grad_centers(batch, targets)
        gv, _, gf = batch.backward(gc)
        for trial in range(3):
            du, df = _direction(batch, v0, f0, rng)
            for w in range(len(seeds)):
                adjoint = float((gv[w].astype(np.float64) * du[w]).sum() + (gf[w].astype(np.float64) * df[w]).sum())
                tl = _tangent_derivative(tangent, batch, w, du, df, gc)
                assert abs(adjoint - tl) <= 1e-3 * max(abs(tl), 1e-6), (steps, flags, w, trial, adjoint, tl)


@pytest.mark.parametrize("flags", [0, B.NO_RECYCLING, B.NO_WARM_STARTING])
def test_adjoint_matches_tangent_linear_without_recycling_or_warm_start(gpu_lib, tangent, flags):
    batch, targets = _make(gpu_lib, [444], flags=flags)
    rng = np.random.default_rng(flags)
    with batch:
        v0, f0 = batch.velocities(), batch.friction()
        _run(batch, v0, f0, 40)
        _, gc = _loss_and_grad_centers(batch, targets)
        gv, _, gf = batch.backward(gc)
        du, df = _direction(batch, v0, f0, rng)
        adjoint = float((gv[0].astype(np.float64) * du[0]).sum() + (gf[0].astype(np.float64) * df[0]).sum())
        tl = _tangent_derivative(tangent, batch, 0, du, df, gc)
        assert abs(adjoint - tl) <= 1e-3 * max(abs(tl), 1e-6), (flags, adjoint, tl)


def test_adjoint_matches_finite_differences(gpu_lib):
    """Central differences of a linear functional of the final centers over 2 steps."""
    seeds = [777, 778]
    steps = 2
    batch, _ = _make(gpu_lib, seeds, 4, 4)
    rng = np.random.default_rng(5)
    with batch:
        v0, f0 = batch.velocities(), batch.friction()
        weights = [rng.standard_normal((s.body_count, 2)).astype(np.float32) * batch.dynamic_masks[w][:, None]
                   for w, s in enumerate(batch.scenes)]

        def functional():
            return sum(float((c.astype(np.float64) * wt).sum()) for c, wt in zip(batch.centers(), weights))

        _run(batch, v0, f0, steps)
        gv, _, gf = batch.backward(weights)
        du, df = _direction(batch, v0, f0, rng)
        adjoint = sum(float((gv[w] * du[w]).sum() + (gf[w] * df[w]).sum()) for w in range(len(seeds)))
        h = 1e-3
        _run(batch, [v + h * d for v, d in zip(v0, du)], [f + h * d for f, d in zip(f0, df)], steps)
        lp = functional()
        _run(batch, [v - h * d for v, d in zip(v0, du)], [f - h * d for f, d in zip(f0, df)], steps)
        lm = functional()
        fd = (lp - lm) / (2 * h)
        assert abs(adjoint - fd) <= 2e-2 * max(abs(fd), 1e-3), (adjoint, fd)


def test_adjoint_matches_finite_differences_in_a_smooth_regime(gpu_lib):
    """One box on the ramp for 5 steps: the perturbation takes no other branch of the step
    (contact, clip, friction cone), so central differences (h = 1e-2) of the forward step
    resolve the derivative; the adjoint must match them to 1e-3 along a velocity direction,
    a velocity-and-friction direction and a linear-velocity-only direction."""
    batch, _ = _make(gpu_lib, [777], 1, 1)
    rng = np.random.default_rng(5)
    steps, h = 5, 1e-2
    with batch:
        v0, f0 = batch.velocities(), batch.friction()
        weights = [rng.standard_normal((s.body_count, 2)).astype(np.float32) * batch.dynamic_masks[w][:, None]
                   for w, s in enumerate(batch.scenes)]

        def functional():
            return sum(float((c.astype(np.float64) * wt).sum()) for c, wt in zip(batch.centers(), weights))

        for kind in ("velocity", "velocity and friction", "linear velocity"):
            du = [rng.standard_normal(v.shape).astype(np.float32) * batch.dynamic_masks[w][:, None] for w, v in enumerate(v0)]
            if kind == "linear velocity":
                for d in du:
                    d[:, 2] = 0.0
            scale = 1.0 if kind == "velocity and friction" else 0.0
            df = [rng.standard_normal(f.shape).astype(np.float32) * scale for f in f0]
            for f in df:
                f[0] = 0.0
            _run(batch, v0, f0, steps)
            gv, _, gf = batch.backward(weights)
            adjoint = float((gv[0].astype(np.float64) * du[0]).sum() + (gf[0].astype(np.float64) * df[0]).sum())
            _run(batch, [v + h * d for v, d in zip(v0, du)], [f + h * d for f, d in zip(f0, df)], steps)
            lp = functional()
            _run(batch, [v - h * d for v, d in zip(v0, du)], [f - h * d for f, d in zip(f0, df)], steps)
            lm = functional()
            fd = (lp - lm) / (2 * h)
            assert abs(adjoint - fd) <= 1e-3 * abs(fd), (kind, adjoint, fd)


def test_torch_autograd_function(gpu_lib):
    """The torch.autograd.Function over the C ABI gives the adjoint's gradients."""
    torch = pytest.importorskip("torch")
    from box2d_gb300.diff import make_step_function

    batch, targets = _make(gpu_lib, [31, 32], 4, 4)
    with batch:
        v0 = torch.tensor(np.stack(batch.velocities()), requires_grad=True)
        f0 = torch.tensor(np.stack(batch.friction()), requires_grad=True)
        StepBatch = make_step_function()
        centers = StepBatch.apply(v0, f0, batch, 10, 1.0 / 60.0, 4)
        com = centers[:, 1:].double().mean(1)
        loss = ((com - torch.tensor(targets)) ** 2).sum()
        loss.backward()
        _, gc = _loss_and_grad_centers(batch, targets)
        gv, _, gf = batch.backward(gc)
        assert np.allclose(v0.grad.numpy(), np.stack(gv), rtol=1e-5, atol=1e-8)
        assert np.allclose(f0.grad.numpy(), np.stack(gf), rtol=1e-5, atol=1e-8)
        assert float(loss.detach()) > 0.0
