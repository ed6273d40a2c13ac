"""GB300 (sm_103a) implementation of Box2D v3.2's per-step hot path behind the Box2D C API.

The product is the shared library ``libbox2d_gb300.so`` in this directory: it exports the
``box2d.h`` subset declared in ``include/box2d_gb300.h`` (b2CreateWorld, b2World_Step,
bodies, shapes, joints, events) and runs the step on the GPU. This module only locates
and loads it with ctypes, plus the scene builders compiled into it (``b2s_*``) and the
parity probes (``b2p_*``). There is no CPU path: if the library or a CUDA device is
missing, loading or world creation fails loudly.
"""
from __future__ import annotations

import ctypes
from pathlib import Path

import numpy as np

PKG_DIR = Path(__file__).resolve().parent
LIB_PATH = PKG_DIR / "libbox2d_gb300.so"

# scene kinds of scenes.c
LARGE_PYRAMID = 0
MANY_PYRAMIDS_RAIN = 1
JOINT_GRID_MIXED = 2
BATCH_WORLD = 3
RAMP_WORLD = 4
MANY_PYRAMIDS_REF = 5
JOINT_GRID_REF = 6
HELLO_WORLD = 7
SHAPE_ZOO = 8
JOINT_ZOO = 9
FALLING_HINGES = 10
SLEEP_PYRAMIDS = 11
JOINT_MIX = 12
OVERFLOW = 13
SENSOR_ZOO = 14
CHAIN_ZOO = 15
BULLET_ZOO = 16

# scripted body changes (Scene.apply): name -> b2s_body_action kind
BODY_ACTIONS = {"force": 0, "force_center": 1, "torque": 2, "impulse": 3, "impulse_center": 4, "angular_impulse": 5,
                "transform": 6, "target": 7, "destroy_body": 8, "destroy_shape": 9}

NO_CONTINUOUS = 1
NO_WARM_STARTING = 2
NO_RECYCLING = 4
ROLLING_RESISTANCE = 8  # ramp world: rounded boxes with rolling resistance
BALLS = 16  # ramp world: every other body a ball
CAPSULES = 32  # ramp world: two capsules at the ends of the bottom row
SEGMENT_RAMP = 64  # ramp world: the ramp's top face is a segment shape


class WorldId(ctypes.Structure):
    """b2WorldId (id.h): world slot + 1 and generation, passed by value."""
    _fields_ = [("index1", ctypes.c_uint16), ("generation", ctypes.c_uint16)]

    @classmethod
    def unpack(cls, packed: int) -> "WorldId":
        return cls(packed >> 16, packed & 0xFFFF)


def _bind(lib: ctypes.CDLL) -> ctypes.CDLL:
    c_int, c_u32, c_u64, c_f, c_p = ctypes.c_int, ctypes.c_uint32, ctypes.c_uint64, ctypes.c_float, ctypes.c_void_p
    sig = {
        "b2s_create": (c_int, [c_int, c_int, c_int, c_int, c_u32, c_int]),
        "b2s_destroy": (None, [c_int]),
        "b2s_step": (None, [c_int, c_f, c_int, c_int]),
        "b2s_step_batch": (None, [c_p, c_int, c_f, c_int, c_int, c_int]),
        "b2s_body_count": (c_int, [c_int]),
        "b2s_dynamic_count": (c_int, [c_int]),
        "b2s_world_id": (c_u32, [c_int]),
        "b2s_get_state": (None, [c_int, c_p]),
        "b2s_move_events": (c_int, [c_int, c_p, c_int]),
        "b2s_move_events_many": (c_int, [c_p, c_int, c_p, c_int]),
        "b2s_state_hash": (c_u64, [c_int]),
        "b2s_set_velocities": (None, [c_int, c_p]),
        "b2s_target": (None, [c_int, c_p]),
        "b2s_counters": (None, [c_int, c_p]),
        "b2s_run_until_asleep": (c_int, [c_int, c_int, c_p]),
        "b2s_awake": (c_int, [c_int, c_p]),
        "b2p_contacts": (c_int, [c_u32, c_p, c_int]),
        "b2p_contact_floats": (c_int, [c_u32, c_p, c_int]),
    }
    optional = {
        "b2s_set_body_velocity": (None, [c_int, c_int, c_f, c_f, c_f]),
        "b2s_set_workers": (None, [c_int]),
        "b2s_body_action": (None, [c_int, c_int, c_int, c_f, c_f, c_f, c_f]),
        "b2s_contact_events": (c_int, [c_int, c_p, c_int]),
        "b2s_world_state_hash": (c_u64, [c_int]),
        "b2s_sensor_events": (c_int, [c_int, c_p, c_int]),
        "b2s_set_awake": (None, [c_int, c_int, c_int]),
        "b2s_snapshot": (c_int, [c_int]),
        "b2s_restore": (c_int, [c_int]),
        "b2s_from_snapshot": (c_int, [c_int]),
        "b2s_add_box": (c_int, [c_int, c_f, c_f]),
        "b2s_body_valid": (c_int, [c_int, c_int]),
        "b2World_Snapshot": (c_int, [WorldId, c_p, c_int]),
        "b2World_Restore": (ctypes.c_bool, [WorldId, c_p, c_int]),
        "b2CreateWorldFromSnapshot": (WorldId, [c_p, c_int, c_int]),
        "b2World_GetStateHash": (c_u64, [WorldId]),
        "b2World_IsValid": (ctypes.c_bool, [WorldId]),
        "b2s_enable_sleep": (None, [c_int, c_int]),
        "b2p_timings": (c_int, [c_u32, c_p, c_p, c_int]),
        "b2p_stream": (c_p, [c_u32]),
        "b2p_status": (c_int, [c_u32]),
        "b2p_host_profile": (c_int, [c_u32, c_p, c_int]),
        "b2p_contacts_noalloc": (c_int, [c_u32, c_p, c_int]),
        "b2p_continuous_counts": (None, [c_u32, c_p]),
        "b2s_set_friction": (None, [c_int, c_p, c_int]),
        "b2s_get_friction": (None, [c_int, c_p, c_int]),
        "b2s_get_centers": (None, [c_int, c_p]),
        "b2s_body_ids": (None, [c_int, c_p]),
        "b2p_batch_profile": (None, [c_p, c_int]),
        "b2Diff_CreateTape": (c_p, [c_p, c_int]),
        "b2Diff_DestroyTape": (None, [c_p]),
        "b2Diff_Record": (None, [c_p, ctypes.c_bool]),
        "b2Diff_StepCount": (c_int, [c_p]),
        "b2Diff_Backward": (c_int, [c_p, c_p, c_p, c_p, c_p, c_p, c_p]),
        "b2Diff_Sizes": (None, [c_p, c_p, c_p]),
        "b2Diff_LastBackwardMs": (c_f, [c_p, c_p]),
        "b2Diff_LastFailure": (None, [c_p, c_p]),
        "b2Diff_DownloadTape": (ctypes.c_longlong, [c_p, c_int, c_p, ctypes.c_longlong]),
    }
    for name, (res, args) in optional.items():
        if hasattr(lib, name):
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
    for name, (res, args) in sig.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    return lib


def load_library(path: str | Path | None = None) -> ctypes.CDLL:
    """Load a Box2D-API shared library (the GB300 library by default) with its scene and
    probe entry points bound. Raises if the file is missing."""
    p = Path(path) if path is not None else LIB_PATH
    if not p.exists():
        raise FileNotFoundError(
            f"{p} is missing: build it with `python -c \"import __graft_entry__ as g; g.build()\"` "
            "(the GB300 step library has no CPU fallback)")
    return _bind(ctypes.CDLL(str(p)))


class Scene:
    """A world built by one of the scene builders, stepped through the public C API."""

    def __init__(self, lib: ctypes.CDLL, kind: int, a: int = 0, b: int = 0, c: int = 0, seed: int = 0, flags: int = 0):
        self.lib = lib
        self.handle = lib.b2s_create(kind, a, b, c, seed, flags)
        if self.handle < 0:
            raise RuntimeError("scene creation failed (no world slot, or no usable CUDA device for the GB300 library)")
        self.body_count = lib.b2s_body_count(self.handle)
        self.dynamic_count = lib.b2s_dynamic_count(self.handle)

    @classmethod
    def _from_handle(cls, lib: ctypes.CDLL, handle: int) -> "Scene":
        scene = cls.__new__(cls)
        scene.lib = lib
        scene.handle = handle
        scene.body_count = lib.b2s_body_count(handle)
        scene.dynamic_count = lib.b2s_dynamic_count(handle)
        return scene

    # ---- snapshots (b2World_Snapshot, b2World_Restore, b2CreateWorldFromSnapshot) ----
    def snapshot(self) -> int:
        """Snapshot the world into an image the scene keeps (with its body list); returns
        the image size."""
        return self.lib.b2s_snapshot(self.handle)

    def restore(self) -> bool:
        """Restore the world (and the body list) from the scene's kept image."""
        ok = self.lib.b2s_restore(self.handle) == 1
        self.body_count = self.lib.b2s_body_count(self.handle)
        return ok

    def from_snapshot(self) -> "Scene":
        """A new scene whose world is created from the kept image."""
        handle = self.lib.b2s_from_snapshot(self.handle)
        if handle < 0:
            raise RuntimeError("b2CreateWorldFromSnapshot failed")
        return Scene._from_handle(self.lib, handle)

    def snapshot_image(self) -> bytes:
        """The world's snapshot image through the public API (size query, then fill)."""
        wid = WorldId.unpack(self.world_id)
        size = self.lib.b2World_Snapshot(wid, None, 0)
        buf = ctypes.create_string_buffer(max(size, 1))
        written = self.lib.b2World_Snapshot(wid, buf, size)
        assert written == size
        return buf.raw[:size]

    def restore_image(self, image: bytes | None) -> bool:
        wid = WorldId.unpack(self.world_id)
        if image is None:
            return bool(self.lib.b2World_Restore(wid, None, 0))
        buf = ctypes.create_string_buffer(image, len(image))
        return bool(self.lib.b2World_Restore(wid, buf, len(image)))

    def add_box(self, x: float, y: float) -> int:
        index = self.lib.b2s_add_box(self.handle, x, y)
        self.body_count = self.lib.b2s_body_count(self.handle)
        return index

    def body_valid(self, index: int) -> bool:
        return self.lib.b2s_body_valid(self.handle, index) == 1

    @property
    def world_id(self) -> int:
        return self.lib.b2s_world_id(self.handle)

    def step(self, count: int = 1, dt: float = 1.0 / 60.0, substeps: int = 4) -> None:
        self.lib.b2s_step(self.handle, dt, substeps, count)

    def state(self) -> np.ndarray:
        out = np.zeros((self.body_count, 7), np.float32)
        self.lib.b2s_get_state(self.handle, out.ctypes.data)
        return out

    def move_events(self, out: np.ndarray | None = None) -> np.ndarray:
        """Transforms (p.x, p.y, q.c, q.s) of the last step's body move events."""
        if out is None or out.shape[0] < self.body_count:
            out = np.zeros((self.body_count, 4), np.float32)
        n = self.lib.b2s_move_events(self.handle, out.ctypes.data, out.shape[0])
        return out[:n]

    def state_hash(self) -> int:
        return int(self.lib.b2s_state_hash(self.handle))

    def world_state_hash(self) -> int:
        """b2World_GetStateHash of the scene's world (libraries that export it)."""
        return int(self.lib.b2s_world_state_hash(self.handle))

    def contacts(self) -> np.ndarray:
        cap = 1 << 16
        while True:
            buf = np.zeros((cap, 8), np.int32)
            n = self.lib.b2p_contacts(self.world_id, buf.ctypes.data, cap)
            if n <= cap:
                return buf[:n]
            cap = n

    def contact_floats(self) -> np.ndarray:
        cap = 1 << 16
        while True:
            buf = np.zeros((cap, 12), np.float32)
            n = self.lib.b2p_contact_floats(self.world_id, buf.ctypes.data, cap)
            if n <= cap:
                return buf[:n]
            cap = n

    def contact_events(self) -> np.ndarray:
        """The last step's contact begin/end touch events, one row each: kind (0 begin,
        1 end), shape A, shape B, contact id, contact generation."""
        cap = 4096
        while True:
            buf = np.zeros((cap, 5), np.int32)
            n = self.lib.b2s_contact_events(self.handle, buf.ctypes.data, cap)
            if n <= cap:
                return buf[:n]
            cap = n

    def sensor_events(self) -> np.ndarray:
        """The last step's sensor begin/end touch events, one row each: kind (0 begin,
        1 end), sensor shape, visitor shape, sensor generation, visitor generation."""
        cap = 4096
        while True:
            buf = np.zeros((cap, 5), np.int32)
            n = self.lib.b2s_sensor_events(self.handle, buf.ctypes.data, cap)
            if n <= cap:
                return buf[:n]
            cap = n

    def timings(self, reset: bool = False) -> tuple[np.ndarray, np.ndarray]:
        """Accumulated device stage times (ms: pairs, narrowphase, solver, finalize) and
        host<->device traffic (bytes: to device, to host) and kernels launched."""
        ms = np.zeros(4, np.float32)
        traffic = np.zeros(3, np.int64)
        self.lib.b2p_timings(self.world_id, ms.ctypes.data, traffic.ctypes.data, int(reset))
        return ms, traffic

    def host_profile(self, reset: bool = False) -> np.ndarray:
        """Accumulated host time per step phase (ms): tree upload, pair query, contact
        creation, tree rebuild, narrowphase, contact-state pass, uploads, solver, proxy
        enlargement, unused."""
        out = np.zeros(10, np.float32)
        self.lib.b2p_host_profile(self.world_id, out.ctypes.data, int(reset))
        return out

    def continuous_counts(self) -> tuple[int, int]:
        """Fast non-bullet bodies swept against static shapes, and sweeps that ended at a
        time of impact, since the world was created."""
        out = np.zeros(2, np.int32)
        self.lib.b2p_continuous_counts(self.world_id, out.ctypes.data)
        return int(out[0]), int(out[1])

    def run_until_asleep(self, step_limit: int = 500) -> tuple[int, int]:
        """Step until no body moves (every island asleep); returns (step count, b2Hash of
        the dynamic bodies' transforms), or (-1, 0) within the limit."""
        out = np.zeros(1, np.uint32)
        n = self.lib.b2s_run_until_asleep(self.handle, step_limit, out.ctypes.data)
        return int(n), int(out[0])

    def apply(self, action: list) -> None:
        """One scripted change between steps: ["velocity", body, vx, vy, w], ["awake", body,
        flag], ["sleeping", flag], ["snapshot"], ["restore"], or a body action of BODY_ACTIONS with its body index and up
        to four numbers (see b2s_body_action)."""
        kind = action[0]
        if kind == "velocity":
            self.lib.b2s_set_body_velocity(self.handle, int(action[1]), float(action[2]), float(action[3]),
                                           float(action[4]))
        elif kind == "awake":
            self.lib.b2s_set_awake(self.handle, int(action[1]), int(action[2]))
        elif kind == "sleeping":
            self.lib.b2s_enable_sleep(self.handle, int(action[1]))
        elif kind == "snapshot":
            if self.snapshot() <= 0:
                raise RuntimeError("b2World_Snapshot failed")
        elif kind == "restore":
            if not self.restore():
                raise RuntimeError("b2World_Restore refused the scene's image")
        elif kind in BODY_ACTIONS:
            args = [float(x) for x in action[2:]] + [0.0] * (4 - len(action[2:]))
            self.lib.b2s_body_action(self.handle, BODY_ACTIONS[kind], int(action[1]), *args[:4])
        else:
            raise ValueError(f"unknown scene action {kind!r}")

    def awake(self) -> tuple[int, np.ndarray]:
        """Awake body count of the world and the awake flag of each scene body."""
        flags = np.zeros(self.body_count, np.int32)
        n = self.lib.b2s_awake(self.handle, flags.ctypes.data)
        return int(n), flags

    def counters(self) -> np.ndarray:
        out = np.zeros(30, np.int32)
        self.lib.b2s_counters(self.handle, out.ctypes.data)
        return out

    def close(self) -> None:
        if self.handle >= 0:
            self.lib.b2s_destroy(self.handle)
            self.handle = -1

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()
