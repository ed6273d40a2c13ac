"""Differentiable batched stepping (box2d_gb300_diff.h) through the C ABI, and a
torch.autograd.Function over it.

A ``DiffBatch`` holds many worlds built by the scene builders, recorded on one tape. Its
forward pass sets each dynamic body's initial linear and angular velocity and each
shape's friction, steps every world on the GPU (one host thread per group of worlds, one
CUDA stream per world) and returns the final centers of mass; its backward pass runs the
adjoint kernels over every recorded step of every world in one launch per step.
"""
from __future__ import annotations

import ctypes

import numpy as np

import box2d_gb300 as B

DIFF_ERRORS = {
    -1: "a recorded step holds something the adjoint does not differentiate",
    -2: "recomputing a recorded step did not reproduce the recorded result",
    -3: "no step recorded",
    -4: "bad argument",
}


class DiffBatch:
    """Worlds of one scene kind with seeds ``seeds``, stepped together and recorded."""

    def __init__(self, lib: ctypes.CDLL, kind: int, a: int, b: int, c: int, seeds, flags: int = 0):
        if not hasattr(lib, "b2Diff_CreateTape"):
            raise RuntimeError("this library has no differentiable stepping (b2Diff_*)")
        self.lib = lib
        self.spec = (kind, a, b, c, list(seeds), flags)
        self.tape = None
        self.scenes: list[B.Scene] = []
        self._build()

    def _build(self) -> None:
        kind, a, b, c, seeds, flags = self.spec
        self.close()
        self.scenes = [B.Scene(self.lib, kind, a, b, c, s, flags) for s in seeds]
        ids = np.array([[s.world_id >> 16, s.world_id & 0xFFFF] for s in self.scenes], dtype=np.uint16)
        self.tape = self.lib.b2Diff_CreateTape(ids.ctypes.data, len(self.scenes))
        if not self.tape:
            raise RuntimeError("b2Diff_CreateTape failed")
        n = len(self.scenes)
        self.body_counts = np.zeros(n, np.int32)
        self.shape_counts = np.zeros(n, np.int32)
        self.lib.b2Diff_Sizes(self.tape, self.body_counts.ctypes.data, self.shape_counts.ctypes.data)
        self.body_offsets = np.concatenate([[0], np.cumsum(self.body_counts)]).astype(np.int64)
        self.shape_offsets = np.concatenate([[0], np.cumsum(self.shape_counts)]).astype(np.int64)
        self.body_ids = []
        for s in self.scenes:
            ids_ = np.zeros(s.body_count, np.int32)
            self.lib.b2s_body_ids(s.handle, ids_.ctypes.data)
            self.body_ids.append(ids_)

    @property
    def world_count(self) -> int:
        return len(self.scenes)

    def reset(self) -> None:
        """Rebuild every world from its seed (the recorded steps are dropped)."""
        self._build()

    # ---- parameters, in scene body order / shape id order ----
    def velocities(self) -> list[np.ndarray]:
        return [s.state()[:, 4:7].copy() for s in self.scenes]

    def set_velocities(self, v: list[np.ndarray]) -> None:
        for s, vi in zip(self.scenes, v):
            vi = np.ascontiguousarray(vi, np.float32)
            self.lib.b2s_set_velocities(s.handle, vi.ctypes.data)

    def friction(self) -> list[np.ndarray]:
        out = []
        for s, n in zip(self.scenes, self.shape_counts):
            f = np.zeros(int(n), np.float32)
            self.lib.b2s_get_friction(s.handle, f.ctypes.data, int(n))
            out.append(f)
        return out

    def set_friction(self, f: list[np.ndarray]) -> None:
        for s, fi, n in zip(self.scenes, f, self.shape_counts):
            fi = np.ascontiguousarray(fi, np.float32)
            self.lib.b2s_set_friction(s.handle, fi.ctypes.data, int(n))

    def centers(self) -> list[np.ndarray]:
        out = []
        for s in self.scenes:
            c = np.zeros((s.body_count, 2), np.float32)
            self.lib.b2s_get_centers(s.handle, c.ctypes.data)
            out.append(c)
        return out

    # ---- stepping ----
    def step(self, steps: int, dt: float = 1.0 / 60.0, substeps: int = 4, threads: int = 0, record: bool = True) -> None:
        self.lib.b2Diff_Record(self.tape, bool(record))
        handles = np.array([s.handle for s in self.scenes], np.int32)
        self.lib.b2s_step_batch(handles.ctypes.data, len(handles), dt, substeps, steps, threads)
        self.lib.b2Diff_Record(self.tape, False)

    def step_count(self) -> int:
        return int(self.lib.b2Diff_StepCount(self.tape))

    def backward(self, grad_centers: list[np.ndarray], grad_velocities: list[np.ndarray] | None = None):
        """Adjoint of every recorded step. ``grad_centers[w]`` is dL/d(center) after the last
        step for each scene body of world w; returns dL/d(initial velocity) per scene body
        (3 per body), dL/d(initial center) per scene body (2) and dL/d(friction) per shape id."""
        total = int(self.body_offsets[-1])
        adj_c = np.zeros((total, 2), np.float32)
        adj_v = np.zeros((total, 3), np.float32)
        for w, g in enumerate(grad_centers):
            adj_c[self.body_offsets[w] + self.body_ids[w]] = g
            if grad_velocities is not None:
                adj_v[self.body_offsets[w] + self.body_ids[w]] = grad_velocities[w]
        gv = np.zeros((total, 3), np.float32)
        gc = np.zeros((total, 2), np.float32)
        gf = np.zeros(int(self.shape_offsets[-1]), np.float32)
        rc = self.lib.b2Diff_Backward(self.tape, adj_c.ctypes.data, None, adj_v.ctypes.data, gv.ctypes.data, gc.ctypes.data,
                                      gf.ctypes.data)
        if rc != 0:
            f = np.zeros(5, np.int32)
            self.lib.b2Diff_LastFailure(self.tape, f.ctypes.data)
            raise RuntimeError(f"b2Diff_Backward: {DIFF_ERRORS.get(rc, f'CUDA error {rc}')} "
                               f"(world {f[1]}, step {f[2]}, check {f[3]}, item {f[4]})")
        grad_v = [gv[self.body_offsets[w] + self.body_ids[w]] for w in range(self.world_count)]
        grad_c = [gc[self.body_offsets[w] + self.body_ids[w]] for w in range(self.world_count)]
        grad_f = [gf[self.shape_offsets[w]:self.shape_offsets[w + 1]] for w in range(self.world_count)]
        return grad_v, grad_c, grad_f

    def backward_ms(self) -> tuple[float, int]:
        launches = ctypes.c_int(0)
        ms = self.lib.b2Diff_LastBackwardMs(self.tape, ctypes.byref(launches))
        return float(ms), int(launches.value)

    def download_tape(self, world: int) -> bytes:
        n = self.lib.b2Diff_DownloadTape(self.tape, world, None, 0)
        buf = np.zeros(int(n), np.uint8)
        got = self.lib.b2Diff_DownloadTape(self.tape, world, buf.ctypes.data, int(n))
        if got != n:
            raise RuntimeError("b2Diff_DownloadTape failed")
        return buf.tobytes()

    def close(self) -> None:
        if self.tape:
            self.lib.b2Diff_DestroyTape(self.tape)
            self.tape = None
        for s in self.scenes:
            s.close()
        self.scenes = []

    def __enter__(self):
        return self

    def __exit__(self, *exc) -> None:
        self.close()


def make_step_function():
    """``StepBatch.apply(v0, friction, batch, steps, dt, substeps)``: a torch.autograd.Function
    whose forward rebuilds ``batch``, sets the initial velocities ``v0`` [W, bodies, 3] (scene
    body order) and frictions ``friction`` [W, shapes] (shape id order), steps it and returns
    the final centers of mass [W, bodies, 2]; its backward runs the adjoint kernels."""
    import torch

    class StepBatch(torch.autograd.Function):
        @staticmethod
        def forward(ctx, v0, friction, batch: DiffBatch, steps: int, dt: float, substeps: int):
            batch.reset()
            batch.set_velocities([v.detach().cpu().numpy() for v in v0])
            batch.set_friction([f.detach().cpu().numpy() for f in friction])
            batch.step(steps, dt, substeps)
            ctx.batch = batch
            ctx.device = v0.device
            return torch.from_numpy(np.stack(batch.centers())).to(v0.device)

        @staticmethod
        def backward(ctx, grad_centers):
            g = grad_centers.detach().cpu().numpy().astype(np.float32)
            gv, _, gf = ctx.batch.backward([g[w] for w in range(g.shape[0])])
            return (torch.from_numpy(np.stack(gv)).to(ctx.device), torch.from_numpy(np.stack(gf)).to(ctx.device),
                    None, None, None, None)

    return StepBatch
