"""Shared fixtures. Tests marked `gpu` need a CUDA device and the built GB300 library;
everything else runs on CPU (the oracle, the golden fixtures, the ABI checks)."""
from __future__ import annotations

import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))

import box2d_gb300 as B  # noqa: E402

GOLDEN = ROOT / "tests" / "golden"
ORACLE_LIB = ROOT / "oracle" / "liboracle.so"
REF_LIB = ROOT / "oracle" / "_ref" / "libref.so"


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


@pytest.fixture(scope="session")
def gpu_lib():
    """The GB300 library; fails (does not skip) when it is missing on a GPU run."""
    return B.load_library()
