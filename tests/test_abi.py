"""The C ABI: the GB300 library loads on CPU-only machines and exports every function
declared in include/*.h; the public structs have the reference's layout (checked by
compiling a layout probe against the reference headers where they are present)."""
from __future__ import annotations

import ctypes
import re
import subprocess
import tempfile
from pathlib import Path

import pytest

import box2d_gb300 as B
from conftest import reference_dir

ROOT = Path(__file__).resolve().parents[1]


def declared_functions() -> set[str]:
    """Every exported function prototype of include/*.h (B2G_API lines of the public
    header, plain prototypes of the probe header)."""
    names = set()
    for h in (ROOT / "include").glob("*.h"):
        for line in h.read_text().splitlines():
            m = re.match(r"^B2G_API\s+[\w\s\*]+?\b(b2\w+)\s*\(", line) or \
                re.match(r"^(?:int|void|float|uint32_t|uint64_t)\s+\**(b2\w+)\s*\(", line)
            if m:
                names.add(m.group(1))
    return names


def test_library_exports_every_declared_function():
    if not B.LIB_PATH.exists():
        import box2d_gb300._build as bld
        bld.build_library()
    lib = ctypes.CDLL(str(B.LIB_PATH))
    missing = [n for n in sorted(declared_functions()) if not hasattr(lib, n)]
    assert not missing, f"declared but not exported: {missing}"
    assert len(declared_functions()) > 80


def test_oracle_exports_the_public_api(oracle):
    skip = {"b2p_status", "b2p_timings", "b2p_stream", "b2p_host_profile", "b2p_contacts_noalloc", "b2World_StepBatch",
            "b2p_batch_profile",
            # islands and sleeping are pinned against fixtures of the reference itself
            # (tests/golden/make_golden.py), not restated in the oracle
            "b2Body_SetAwake", "b2Body_GetSleepThreshold",
            # the state hash covers island and solver-set bookkeeping the oracle does not
            # restate; the GB300 library is checked against the reference's values directly
            "b2World_GetStateHash", "b2s_world_state_hash", "b2p_state_words",
            # sensors are checked against fixtures recorded from the reference itself
            "b2World_GetSensorEvents", "b2Shape_IsSensor", "b2Shape_EnableSensorEvents",
            "b2Shape_AreSensorEventsEnabled", "b2Shape_GetSensorCapacity", "b2Shape_GetSensorData",
            "b2s_sensor_events",
            # chain shapes are checked against fixtures recorded from the reference itself
            "b2DefaultChainDef", "b2CreateChain", "b2Chain_IsValid", "b2Chain_GetSegmentCount", "b2Chain_GetSegments",
            "b2CreateChainSegmentShape", "b2Shape_GetType", "b2Shape_GetChainSegment", "b2Shape_GetParentChain",
            "b2DestroyChain",
            # destruction changes island and solver-set bookkeeping the oracle does not restate;
            # checked against fixtures recorded from the reference itself
            "b2DestroyBody", "b2DestroyShape", "b2DestroyJoint",
            # snapshots hold the library's own bookkeeping; checked by restoring into the
            # library and stepping against fixtures recorded from the reference
            "b2World_Snapshot", "b2World_Restore", "b2CreateWorldFromSnapshot",
            "b2Shape_IsValid", "b2Joint_IsValid", "b2Shape_GetAABB"}
    # differentiable stepping (box2d_gb300_diff.h) is an extension of the GB300 library; its
    # checker is the host tangent-linear code, not the oracle's public API
    missing = [n for n in sorted(declared_functions())
               if n not in skip and not n.startswith("b2Diff_") and not hasattr(oracle, n)]
    assert not missing, missing


_REF = reference_dir()
REF_INCLUDE = _REF / "include" if _REF else ROOT / "baseline" / "_ref" / "include"


@pytest.mark.skipif(not REF_INCLUDE.is_dir(), reason="reference headers not present on this machine")
def test_struct_layouts_match_reference():
    """Compile one program against the reference headers and one against ours; both print
    sizeof/offsetof of every public struct the API passes by value or pointer."""
    structs = {
        "b2WorldDef": ["gravity", "frictionCallback", "enableSleep", "workerCount", "userData", "capacity", "internalValue"],
        "b2BodyDef": ["type", "position", "rotation", "linearVelocity", "name", "userData", "motionLocks", "enableSleep",
                      "enableContactRecycling", "internalValue"],
        "b2ShapeDef": ["userData", "material", "density", "filter", "enableCustomFiltering", "updateBodyMass",
                       "internalValue"],
        "b2Polygon": ["vertices", "normals", "centroid", "radius", "count"],
        "b2Manifold": ["normal", "rollingImpulse", "points", "pointCount"],
        "b2ManifoldPoint": ["anchorA", "separation", "normalVelocity", "id", "persisted"],
        "b2RevoluteJointDef": ["base", "targetAngle", "enableSpring", "lowerAngle", "enableMotor", "motorSpeed",
                               "internalValue"],
        "b2PrismaticJointDef": ["base", "enableSpring", "targetTranslation", "maxMotorForce", "internalValue"],
        "b2WeldJointDef": ["base", "linearHertz", "angularDampingRatio", "internalValue"],
        "b2WheelJointDef": ["base", "enableSpring", "lowerTranslation", "motorSpeed", "internalValue"],
        "b2DistanceJointDef": ["base", "length", "enableSpring", "maxLength", "motorSpeed", "internalValue"],
        "b2JointDef": ["userData", "bodyIdA", "localFrameA", "forceThreshold", "drawScale", "collideConnected"],
        "b2BodyMoveEvent": ["userData", "transform", "bodyId", "fellAsleep"],
        "b2ContactBeginTouchEvent": ["shapeIdA", "shapeIdB", "contactId"],
        "b2ContactEvents": ["beginEvents", "endEvents", "hitEvents", "beginCount", "hitCount"],
        "b2Counters": ["byteCount", "colorCounts", "recycledContactCount"],
        "b2Profile": ["step", "solve", "sensors"],
        "b2Capacity": ["contactCount"],
        "b2SurfaceMaterial": ["friction", "userMaterialId", "customColor"],
        "b2Filter": ["categoryBits", "maskBits", "groupIndex"],
        "b2Hull": ["points", "count"],
        "b2ContactId": ["index1", "world0", "padding", "generation"],
        "b2BodyId": ["index1", "world0", "generation"],
    }
    body = ["#include <stdio.h>", "#include <stddef.h>", "int main(void){"]
    for s, fields in structs.items():
        body.append(f'printf("{s} %zu\\n", sizeof({s}));')
        for f in fields:
            body.append(f'printf("{s}.{f} %zu\\n", offsetof({s}, {f}));')
    body.append("return 0;}")
    src = "\n".join(body)
    outs = []
    with tempfile.TemporaryDirectory() as td:
        for name, inc, hdr in (("ref", REF_INCLUDE, "box2d/box2d.h"), ("ours", ROOT / "include", "box2d_gb300.h")):
            c = Path(td) / f"{name}.c"
            c.write_text(f'#include "{hdr}"\n' + src)
            exe = Path(td) / name
            subprocess.run(["gcc", "-std=gnu17", "-I", str(inc), str(c), "-o", str(exe)], check=True)
            outs.append(subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout)
    assert outs[0] == outs[1]


def test_reference_include_path_builds_against_the_library():
    """A program written for the reference ("box2d/box2d.h") compiles unchanged against the
    forwarding header and links against libbox2d_gb300.so; the CPU-side calls it makes
    (defaults, geometry helpers) run without a GPU."""
    if not B.LIB_PATH.exists():
        import box2d_gb300._build as bld
        bld.build_library()
    src = r'''
#include "box2d/box2d.h"
#include <stdio.h>
int main(void)
{
	b2WorldDef wd = b2DefaultWorldDef();
	b2BodyDef bd = b2DefaultBodyDef();
	b2Polygon box = b2MakeBox( 0.5f, 0.25f );
	b2MassData md = b2ComputePolygonMass( &box, 1.0f );
	printf( "%.3f %d %d %.4f\n", wd.gravity.y, (int)bd.type, box.count, md.mass );
	return 0;
}
'''
    with tempfile.TemporaryDirectory() as td:
        c = Path(td) / "app.c"
        c.write_text(src)
        exe = Path(td) / "app"
        subprocess.run(["gcc", "-std=gnu17", "-I", str(ROOT / "include"), str(c), "-o", str(exe), "-L", str(B.PKG_DIR),
                        "-lbox2d_gb300", f"-Wl,-rpath,{B.PKG_DIR}"], check=True)
        out = subprocess.run([str(exe)], capture_output=True, text=True, check=True).stdout.split()
    assert out == ["-10.000", "0", "4", "0.5000"]
