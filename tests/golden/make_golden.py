"""Record golden parity fixtures from the reference itself.

Runs only where the reference sources are present: builds the reference from its own
sources into oracle/_ref (oracle/Makefile, target `ref`), drives it through the scene
builders of box2d_gb300/scenes/scenes.c, and writes, per scene, the FNV-1a hash of every
body's (position, rotation, velocity) after each step plus a digest of the live contact
table (contact id, shape pair, graph color, point count, feature ids, touching) at a few
steps. The committed JSON files are what tests compare the oracle and the GB300 library
against on machines without the reference.

Usage: python tests/golden/make_golden.py [scene names]   (all scenes without names)
"""
from __future__ import annotations

import hashlib
import json
import subprocess
import sys
from pathlib import Path

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

import box2d_gb300 as B  # noqa: E402

# (name, kind, a, b, c, seed, flags, steps, contact digest steps)
SCENES = [
    ("large_pyramid_20", B.LARGE_PYRAMID, 20, 0, 0, 0, 0, 300, [1, 10, 100, 300]),
    ("large_pyramid_100_segment", B.LARGE_PYRAMID, 100, 1, 0, 0, 0, 40, [1, 40]),
    ("shape_zoo_200", B.SHAPE_ZOO, 200, 0, 0, 7, B.NO_CONTINUOUS, 300, [1, 50, 300]),
    ("many_pyramids_rain_3x3", B.MANY_PYRAMIDS_RAIN, 3, 10, 100, 0, B.NO_CONTINUOUS, 300, [1, 100, 300]),
    ("joint_grid_20", B.JOINT_GRID_REF, 20, 0, 0, 0, 0, 120, [1, 120]),
    ("joint_grid_mixed_12", B.JOINT_GRID_MIXED, 12, 40, 0, 3, B.NO_CONTINUOUS, 200, [1, 100, 200]),
    ("batch_world_60", B.BATCH_WORLD, 60, 0, 0, 11, B.NO_CONTINUOUS, 200, [1, 200]),
    ("ramp_world_4x4", B.RAMP_WORLD, 4, 4, 0, 5, B.NO_CONTINUOUS, 120, [1, 120]),
    ("joint_zoo_4", B.JOINT_ZOO, 4, 0, 0, 3, B.NO_CONTINUOUS, 300, [1, 150, 300]),
    ("joint_mix_4", B.JOINT_MIX, 4, 0, 0, 5, B.NO_CONTINUOUS, 300, [1, 150, 300]),
    # continuous collision on: fast bodies are swept against static shapes
    ("shape_zoo_200_continuous", B.SHAPE_ZOO, 200, 0, 0, 7, 0, 300, [1, 150, 300]),
    ("many_pyramids_rain_3x3_continuous", B.MANY_PYRAMIDS_RAIN, 3, 10, 100, 0, 0, 300, [1, 150, 300]),
    ("batch_world_continuous", B.BATCH_WORLD, 0, 0, 0, 21, 0, 300, [1, 300]),
    # more constraints on one body than the graph has colors: the overflow color (23) holds
    # contacts and joints, solved by the overflow path
    ("overflow_2", B.OVERFLOW, 2, 0, 0, 4, 0, 240, [1, 60, 240]),
    # forces, torques, impulses, teleports and target transforms applied between steps
    ("body_api_zoo", B.SHAPE_ZOO, 60, 0, 0, 9, 0, 150, [1, 75, 150]),
    # sensors: begin/end overlap events of static, kinematic and dynamic sensor shapes
    ("sensor_zoo_60", B.SENSOR_ZOO, 60, 0, 0, 5, B.NO_CONTINUOUS, 240, [1, 120, 240]),
    ("sensor_zoo_60_continuous", B.SENSOR_ZOO, 60, 0, 0, 6, 0, 240, [1, 120, 240]),
    # shapes dropped from high up cross the thin gate within one step: continuous sensor hits
    ("sensor_gate_120", B.SENSOR_ZOO, 120, 0, 0, 8, 0, 120, [1, 60, 120]),
]

# chain shapes (one-sided segments with ghost vertices), with continuous collision on and
# off; the oracle does not restate chains, so only the GB300 library is checked against these
CHAIN_SCENES = [
    ("chain_zoo_80", B.CHAIN_ZOO, 80, 0, 0, 3, 0, 300, [1, 100, 300]),
    ("chain_zoo_80_discrete", B.CHAIN_ZOO, 80, 0, 0, 4, B.NO_CONTINUOUS, 300, [1, 150, 300]),
]

# bullets swept against dynamic bodies; the oracle advances bullets like other fast bodies
# (static sweeps only), so only the GB300 library is checked against these
BULLET_SCENES = [
    ("bullet_zoo_24", B.BULLET_ZOO, 24, 0, 0, 7, 0, 200, [1, 20, 200]),
]

# sleeping on: islands fall asleep and wake; per step also the awake body count. The
# oracle does not restate islands, so only the GB300 library is checked against these.
SLEEP_SCENES = [
    ("falling_hinges", B.FALLING_HINGES, 0, 0, 0, 0, 0, 300, [1, 100, 274, 300]),
    ("sleep_pyramids_3x8", B.SLEEP_PYRAMIDS, 3, 8, 80, 0, 0, 700, [1, 200, 400, 700]),
    ("sleep_api_pyramids", B.SLEEP_PYRAMIDS, 2, 6, 1000, 0, 0, 330, [1, 56, 131, 201, 330]),
    # bodies and shapes destroyed between steps, awake and asleep
    ("destroy_pyramids", B.SLEEP_PYRAMIDS, 2, 6, 1000, 0, 0, 300, [1, 60, 160, 300]),
    ("destroy_joint_zoo", B.JOINT_ZOO, 4, 0, 0, 3, 0, 200, [1, 50, 100, 200]),
]
# snapshots taken and restored between steps (b2World_Snapshot / b2World_Restore), with
# changes made between them that the restore rolls back; per step also the awake count.
# The oracle does not restate snapshots, so only the GB300 library is checked against these.
SNAPSHOT_SCENES = [
    ("snapshot_sleep_pyramids", B.SLEEP_PYRAMIDS, 2, 6, 1000, 0, 0, 300, [1, 96, 141, 221, 300]),
    ("snapshot_joint_zoo", B.JOINT_ZOO, 4, 0, 0, 3, 0, 200, [1, 61, 141, 200]),
    ("snapshot_sensor_zoo", B.SENSOR_ZOO, 60, 0, 0, 6, 0, 160, [1, 91, 160]),
    ("snapshot_chain_zoo", B.CHAIN_ZOO, 80, 0, 0, 3, 0, 200, [1, 101, 200]),
]
# changes applied after the given step (Scene.apply): wake by velocity, put an island to
# sleep and wake one through b2Body_SetAwake, switch sleeping off and on again
SCRIPTS = {
    "sleep_api_pyramids": [[40, "velocity", 3, 0.0, 6.0, 0.0], [41, "velocity", 25, 2.0, 0.0, 1.0],
                           [55, "awake", 10, 0], [130, "awake", 30, 1], [200, "sleeping", 0], [260, "sleeping", 1]],
}
SCRIPTS["destroy_pyramids"] = [[20, "destroy_body", 3], [40, "destroy_shape", 7], [120, "destroy_body", 12],
                                [121, "destroy_body", 30], [150, "destroy_shape", 25], [200, "destroy_body", 40]]
SCRIPTS["destroy_joint_zoo"] = [[30, "destroy_body", 5], [31, "destroy_body", 9], [60, "destroy_body", 14],
                                 [61, "destroy_shape", 20], [90, "destroy_body", 2]]
SCRIPTS["snapshot_sleep_pyramids"] = [[95, "snapshot"], [100, "velocity", 3, 0.0, 6.0, 0.0], [110, "destroy_body", 12],
                                       [140, "restore"], [170, "snapshot"], [175, "impulse_center", 20, 5.0, 10.0],
                                       [220, "restore"], [230, "restore"]]
SCRIPTS["snapshot_joint_zoo"] = [[30, "snapshot"], [31, "impulse_center", 6, 3.0, 8.0], [60, "restore"],
                                  [100, "snapshot"], [101, "destroy_body", 5], [140, "restore"]]
SCRIPTS["snapshot_sensor_zoo"] = [[50, "snapshot"], [51, "impulse_center", 10, 0.0, 20.0], [90, "restore"],
                                   [120, "snapshot"], [121, "destroy_body", 7], [150, "restore"]]
SCRIPTS["snapshot_chain_zoo"] = [[60, "snapshot"], [61, "impulse_center", 10, 4.0, 9.0], [100, "restore"]]
SCRIPTS["body_api_zoo"] = (
    [[5, "force", 3, 50.0, 100.0, 0.1, 0.2], [5, "force_center", 3, -20.0, 0.0], [6, "torque", 4, 30.0],
     [10, "impulse", 5, 2.0, 5.0, 0.1, 0.0], [11, "impulse_center", 6, -3.0, 1.0], [12, "angular_impulse", 7, 2.0],
     [13, "impulse_center", 11, 1.0e5, 0.0], [14, "force", 0, 100.0, 100.0, 0.0, 0.0],
     [20, "transform", 8, 0.0, 12.0, 0.5], [30, "target", 9, 3.0, 5.0, 0.3, 1.0 / 60.0]]
    + [[k, "force_center", 10, 0.0, 40.0] for k in range(40, 61)]
    + [[k, "torque", 12, -5.0] for k in range(50, 56)])

# test/test_determinism.c:21-22
DETERMINISM_SLEEP_STEP = 274
DETERMINISM_HASH = 0xE86690F4


def contact_digest(table) -> str:
    return hashlib.sha256(table.astype("<i4").tobytes()).hexdigest()


class EventDigest:
    """Contact begin/end touch events of every step: per-step counts and one sha256 over
    every step's event rows (kind, shape A, shape B, contact id, generation) in order."""

    def __init__(self):
        self.h = hashlib.sha256()
        self.begin, self.end = [], []

    def add(self, events) -> None:
        self.h.update(len(events).to_bytes(4, "little"))
        self.h.update(events.astype("<i4").tobytes())
        self.begin.append(int((events[:, 0] == 0).sum()))
        self.end.append(int((events[:, 0] == 1).sum()))

    def record(self) -> dict:
        return {"sha256": self.h.hexdigest(), "begin_per_step": self.begin, "end_per_step": self.end}


def main() -> None:
    subprocess.run(["make", "-s", "-C", str(ROOT / "oracle"), "ref"], check=True)
    ref = B.load_library(ROOT / "oracle" / "_ref" / "libref.so")
    only = set(sys.argv[1:])
    for name, kind, a, b, c, seed, flags, steps, digest_steps in (SCENES + CHAIN_SCENES + BULLET_SCENES + SLEEP_SCENES
                                                                   + SNAPSHOT_SCENES):
        if only and name not in only:
            continue
        entry = (name, kind, a, b, c, seed, flags, steps, digest_steps)
        sleeping = entry in SLEEP_SCENES or entry in SNAPSHOT_SCENES
        script = SCRIPTS.get(name, [])
        with B.Scene(ref, kind, a, b, c, seed, flags) as s:
            hashes, digests, awake, world_hashes = [], {}, [], []
            events = EventDigest()
            sensor_events = EventDigest()
            for k in range(1, steps + 1):
                s.step()
                events.add(s.contact_events())
                sensor_events.add(s.sensor_events())
                for action in script:
                    if action[0] == k:
                        s.apply(action[1:])
                hashes.append(f"{s.state_hash():016x}")
                world_hashes.append(f"{s.world_state_hash():016x}")
                if sleeping:
                    awake.append(s.awake()[0])
                if k in digest_steps:
                    table = s.contacts()
                    digests[str(k)] = {"count": int(table.shape[0]), "sha256": contact_digest(table),
                                       "touching": int(table[:, 7].sum()) if len(table) else 0}
            data = {"scene": name, "kind": kind, "a": a, "b": b, "c": c, "seed": seed, "flags": flags,
                    "dt": 1.0 / 60.0, "substeps": 4, "bodies": s.body_count, "state_hashes": hashes,
                    "contact_digests": digests, "contact_events": events.record(),
                    "sensor_events": sensor_events.record(),
                    "world_state_hashes": world_hashes,
                    "source": "reference built from its own sources (oracle/Makefile ref)"}
            if (name, kind, a, b, c, seed, flags, steps, digest_steps) in CHAIN_SCENES:
                data["requires"] = "chains"
            if (name, kind, a, b, c, seed, flags, steps, digest_steps) in BULLET_SCENES:
                data["requires"] = "bullets"
            if sleeping:
                data["requires"] = "islands"
                data["awake_counts"] = awake
            if entry in SNAPSHOT_SCENES:
                data["requires"] = "snapshots"
            if script:
                data["script"] = script
        if kind == B.FALLING_HINGES:
            # the reference's own determinism test, rerun here: it must give the test's constants
            with B.Scene(ref, kind, a, b, c, seed, flags) as s:
                sleep_step, digest = s.run_until_asleep(500)
            assert (sleep_step, digest) == (DETERMINISM_SLEEP_STEP, DETERMINISM_HASH), (sleep_step, hex(digest))
            data["run_until_asleep"] = {"sleep_step": sleep_step, "hash": f"{digest:08x}"}
        (Path(__file__).parent / f"{name}.json").write_text(json.dumps(data, indent=1))
        print(name, steps, "steps", s.body_count, "bodies")


if __name__ == "__main__":
    main()
