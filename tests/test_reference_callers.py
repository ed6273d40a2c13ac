"""The reference's own caller code builds unchanged against this library's headers and
links against libbox2d_gb300.so: shared/determinism.c (the falling-hinges scene of the
reference's determinism test) with a small driver written here in the manner of
test/test_determinism.c:28-60. On a GPU the program runs and must reproduce the reference
test's constants (sleep step 274, hash 0xE86690F4, test/test_determinism.c:21-22).

The reference sources come from B2G_REFERENCE_DIR or the git-ignored copy staged by the
oracle Makefile (`make -C oracle stage`); the tests skip where neither exists."""
from __future__ import annotations

import subprocess
from pathlib import Path

import pytest

import box2d_gb300 as B
from conftest import reference_dir

ROOT = Path(__file__).resolve().parents[1]

DRIVER = r"""
#include "determinism.h"
#include "box2d/box2d.h"
#include <stdio.h>

int main( void )
{
	b2WorldDef def = b2DefaultWorldDef();
	b2WorldId world = b2CreateWorld( &def );
	if ( B2_IS_NULL( world ) ) return 2;
	FallingHingeData data = CreateFallingHinges( world );
	for ( int i = 0; i < 500; ++i )
	{
		b2World_Step( world, 1.0f / 60.0f, 4 );
		if ( UpdateFallingHinges( world, &data ) ) break;
	}
	printf( "%d 0x%08X\n", data.sleepStep, data.hash );
	DestroyFallingHinges( &data );
	b2DestroyWorld( world );
	return 0;
}
"""


def _build_driver(tmp_path: Path) -> Path:
    ref = reference_dir()
    if ref is None or not (ref / "shared" / "determinism.c").is_file():
        pytest.skip("reference sources not present (set B2G_REFERENCE_DIR or run make -C oracle stage)")
    if not B.LIB_PATH.exists():
        pytest.skip("libbox2d_gb300.so not built")
    main = tmp_path / "driver.c"
    main.write_text(DRIVER)
    exe = tmp_path / "falling_hinges"
    cmd = ["gcc", "-std=gnu17", "-O2", "-ffp-contract=off", "-I", str(ROOT / "include"), "-I", str(ref / "shared"),
           str(main), str(ref / "shared" / "determinism.c"), "-o", str(exe), "-L", str(B.PKG_DIR), "-lbox2d_gb300",
           f"-Wl,-rpath,{B.PKG_DIR}", "-lm"]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr
    return exe


def test_reference_determinism_scene_builds_and_links(tmp_path):
    _build_driver(tmp_path)


@pytest.mark.parametrize("source", ["shared/benchmarks.c", "benchmark/main.c", "test/test_determinism.c"])
def test_reference_benchmark_sources_compile(source):
    """The reference's benchmark scenes (chains, target transforms, the inline math) and its
    benchmark driver compile unchanged against the public headers."""
    ref = reference_dir()
    if ref is None or not (ref / source).is_file():
        pytest.skip("reference sources not present (set B2G_REFERENCE_DIR or run make -C oracle stage)")
    cmd = ["gcc", "-std=gnu17", "-fsyntax-only", "-Werror=implicit-function-declaration", "-I", str(ROOT / "include"),
           "-I", str(ref / "shared"), "-I", str(ref / "test"), str(ref / source)]
    proc = subprocess.run(cmd, capture_output=True, text=True)
    assert proc.returncode == 0, proc.stderr


@pytest.mark.gpu
def test_reference_determinism_scene_runs_to_the_reference_constants(tmp_path):
    exe = _build_driver(tmp_path)
    proc = subprocess.run([str(exe)], capture_output=True, text=True, timeout=300)
    assert proc.returncode == 0, proc.stderr
    sleep_step, digest = proc.stdout.split()
    assert (int(sleep_step), digest) == (274, "0xE86690F4")
