"""Build recipe of the GB300 step library (no cmake).

Compiles the C17 host sources with gcc, the CUDA sources with nvcc for sm_103a, and links
``box2d_gb300/libbox2d_gb300.so`` with the CUDA runtime linked statically. Bit-exact mode
(the default and only mode) compiles device code with --fmad=false, IEEE division and
square root and no flush-to-zero, and host code with -ffp-contract=off, which is how the
reference builds (CMakeLists.txt:53-66).
"""
from __future__ import annotations

import os
import shutil
import subprocess
from concurrent.futures import ThreadPoolExecutor
from pathlib import Path

PKG = Path(__file__).resolve().parent
ROOT = PKG.parent
BUILD = PKG / "_build"
LIB = PKG / "libbox2d_gb300.so"

HOST_SOURCES = ["csrc/host/world.c", "csrc/host/step.c", "csrc/host/joint.c", "csrc/host/tree.c",
                "csrc/host/geometry.c", "csrc/host/probe.c", "csrc/host/batch.c", "csrc/host/diff.c", "csrc/host/island.c",
                "csrc/host/sensor.c", "csrc/host/snapshot.c",
                "scenes/scenes.c"]
# (source, extra nvcc flags). The cluster and persistent solvers read state written by
# other SMs between barriers, so their global loads bypass L1 (-dlcm=cg).
DEVICE_SOURCES = [("csrc/device/world.cu", []), ("csrc/device/components.cu", []),
                  ("csrc/device/cluster.cu", ["-Xptxas", "-dlcm=cg"]), ("csrc/device/noalloc.cu", []),
                  ("csrc/device/persistent.cu", ["-Xptxas", "-dlcm=cg"]),
                  ("csrc/device/adjoint.cu", [])]

NVCC_FLAGS = ["-std=c++17", "-gencode", "arch=compute_103a,code=sm_103a", "-lineinfo", "-O3",
              "--fmad=false", "-prec-div=true", "-prec-sqrt=true", "-ftz=false", "-Xcompiler", "-fPIC",
              "-Xcompiler", "-fvisibility=hidden"]
CFLAGS = ["-std=gnu17", "-O2", "-ffp-contract=off", "-fno-fast-math", "-fPIC", "-fvisibility=hidden", "-Wall",
          "-Wno-unused-function"]


def _nvcc() -> str:
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not Path(cand).exists():
        raise RuntimeError("nvcc not found; the GB300 step library needs the CUDA toolkit to build")
    return cand


def _run(cmd: list[str], cwd: Path | None = None) -> None:
    proc = subprocess.run(cmd, cwd=cwd, capture_output=True, text=True)
    if proc.returncode != 0:
        raise RuntimeError(f"build step failed ({proc.returncode}): {' '.join(cmd)}\n{proc.stdout}\n{proc.stderr}")


def _needs(target: Path, deps: list[Path]) -> bool:
    if not target.exists():
        return True
    t = target.stat().st_mtime
    return any(d.stat().st_mtime > t for d in deps)


def build_library(force: bool = False) -> Path:
    """Compile and link libbox2d_gb300.so; returns its path."""
    BUILD.mkdir(exist_ok=True)
    nvcc = _nvcc()
    include = ["-I", str(ROOT / "include")]
    headers = list((PKG / "csrc").rglob("*.h")) + list((PKG / "csrc").rglob("*.cuh")) + list((ROOT / "include").glob("*.h"))
    jobs = []
    objects = []
    for src in HOST_SOURCES:
        s = PKG / src
        o = BUILD / (src.replace("/", "_") + ".o")
        objects.append(o)
        if force or _needs(o, [s] + headers):
            jobs.append(["gcc", *CFLAGS, "-DB2S_BATCH_API", *include, "-c", str(s), "-o", str(o)])
    for src, extra in DEVICE_SOURCES:
        s = PKG / src
        o = BUILD / (src.replace("/", "_") + ".o")
        objects.append(o)
        if force or _needs(o, [s] + headers):
            jobs.append([nvcc, *NVCC_FLAGS, *extra, *include, "-c", str(s), "-o", str(o)])
    with ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        list(ex.map(_run, jobs))
    if force or jobs or _needs(LIB, objects):
        _run([nvcc, "-shared", "-cudart", "static", "-gencode", "arch=compute_103a,code=sm_103a", "-o", str(LIB),
              *[str(o) for o in objects], "-Xlinker", "-Bsymbolic", "-lm", "-lpthread"])
    return LIB


def build_oracle(with_reference: bool = True) -> None:
    """Build the CPU oracle and, where the reference sources can be found (its checkout, or
    the git-ignored copy the oracle Makefile stages beside the repository), the reference
    itself. The checkout's location comes from the Makefile, or B2G_REFERENCE_DIR."""
    oracle = ROOT / "oracle"
    _run(["make", "-s", "-C", str(oracle), "liboracle.so", "libtangent.so"])
    if with_reference:
        ref = os.environ.get("B2G_REFERENCE_DIR")
        extra = [f"REF={ref}"] if ref else []
        _run(["make", "-s", "-C", str(oracle), "stage", *extra])
        _run(["make", "-s", f"-j{max(2, os.cpu_count() or 2)}", "-C", str(oracle), "ref", *extra])


def build_all(force: bool = False) -> None:
    with ThreadPoolExecutor(max_workers=2) as ex:
        lib = ex.submit(build_library, force)
        orc = ex.submit(build_oracle)
        lib.result()
        orc.result()


if __name__ == "__main__":
    build_all()
    print(LIB)
