"""Shared fixtures. Tests marked `gpu` need a CUDA device and the built GB300 library;
everything else runs on CPU (the oracle, the golden fixtures, the ABI checks)."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import box2d_gb300 as B  # noqa: E402

GOLDEN = ROOT / "tests" / "golden"
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"
REF_LIB = ROOT / "oracle" / "_ref" / "libref.so"


def reference_dir() -> Path | None:
    """The reference's sources: B2G_REFERENCE_DIR when set, else the git-ignored copy the
    oracle Makefile stages (`make stage`) beside the repository; None where neither is."""
    import os

    env = os.environ.get("B2G_REFERENCE_DIR")
    for cand in ([Path(env)] if env else []) + [ROOT / "baseline" / "_ref"]:
        if (cand / "include" / "box2d" / "box2d.h").is_file():
            return cand
    return None


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU and the built libbox2d_gb300.so")


def golden_cases():
    return sorted(p.stem for p in GOLDEN.glob("*.json"))


def load_golden(name: str) -> dict:
    return json.loads((GOLDEN / f"{name}.json").read_text())


@pytest.fixture(scope="session")
def oracle():
    """The CPU oracle library (test checker only), built on demand."""
    if not ORACLE_LIB.exists():
        import box2d_gb300._build as bld
        bld.build_oracle(with_reference=False)
    return B.load_library(ORACLE_LIB)


TANGENT_LIB = ROOT / "oracle" / "libtangent.so"


@pytest.fixture(scope="session")
def tangent():
    """The FP64 tangent-linear checker of the adjoint (test checker only), built on demand."""
    import ctypes

    if not TANGENT_LIB.exists():
        import box2d_gb300._build as bld
        bld.build_oracle(with_reference=False)
    lib = ctypes.CDLL(str(TANGENT_LIB))
    c_p = ctypes.c_void_p
    lib.b2t_tangent.restype = ctypes.c_int
    lib.b2t_tangent.argtypes = [c_p, ctypes.c_longlong, c_p, c_p, c_p, c_p]
    return lib


@pytest.fixture(scope="session")
def gpu_lib():
    """The GB300 library; fails (does not skip) when it is missing on a GPU run."""
    return B.load_library()


class EventCheck:
    """Checks a scene's contact (or sensor) begin/end touch events step by step against a
    fixture's `contact_events` (`sensor_events`) record: per-step counts and one sha256 over
    every step's rows."""

    def __init__(self, g: dict, key: str = "contact_events"):
        import hashlib

        self.rec = g.get(key)
        self.key = key
        self.h = hashlib.sha256()
        self.name = g.get("scene", "")

    def step(self, scene, k: int) -> None:
        if self.rec is None:
            return
        ev = scene.contact_events() if self.key == "contact_events" else scene.sensor_events()
        self.h.update(len(ev).to_bytes(4, "little"))
        self.h.update(ev.astype("<i4").tobytes())
        begin, end = int((ev[:, 0] == 0).sum()), int((ev[:, 0] == 1).sum())
        assert (begin, end) == (self.rec["begin_per_step"][k - 1], self.rec["end_per_step"][k - 1]), \
            f"{self.name}: {self.key} begin/end counts at step {k}"

    def finish(self, steps: int) -> None:
        if self.rec is not None and steps == len(self.rec["begin_per_step"]):
            assert self.h.hexdigest() == self.rec["sha256"], f"{self.name}: {self.key} differ"


def lockstep(gpu_lib, oracle, kind, a, b, c, seed, flags, steps, check_every=1):
    """Step the same scene on the GB300 library and the oracle; every `check_every` steps the
    body states must be bit-identical, and at the end the contact tables too."""
    with B.Scene(gpu_lib, kind, a, b, c, seed, flags) as g, B.Scene(oracle, kind, a, b, c, seed, flags) as o:
        for k in range(1, steps + 1):
            g.step()
            o.step()
            if k % check_every == 0 or k == steps:
                if g.state_hash() != o.state_hash():
                    gs, os_ = g.state(), o.state()
                    bad = np.nonzero((gs.view(np.uint32) != os_.view(np.uint32)).any(1))[0]
                    pytest.fail(f"state differs at step {k} in {len(bad)} bodies, first {bad[:5]}")
        gc, oc = g.contacts(), o.contacts()
        assert gc.shape == oc.shape and (gc == oc).all(), "contact tables differ"
        return g.body_count, gc.shape[0]
