"""The oracle is pinned against the reference: its per-step state hashes and contact
tables must equal the fixtures recorded from the reference build (tests/golden)."""
from __future__ import annotations

import hashlib

import pytest

import box2d_gb300 as B
from conftest import golden_cases, load_golden


@pytest.mark.parametrize("name", golden_cases())
def test_oracle_matches_reference_fixture(oracle, name):
    g = load_golden(name)
    with B.Scene(oracle, g["kind"], g["a"], g["b"], g["c"], g["seed"], g["flags"]) as s:
        assert s.body_count == g["bodies"]
        for k, expected in enumerate(g["state_hashes"], start=1):
            s.step(1, g["dt"], g["substeps"])
            assert f"{s.state_hash():016x}" == expected, f"{name}: state diverged at step {k}"
            d = g["contact_digests"].get(str(k))
            if d is not None:
                table = s.contacts()
                assert table.shape[0] == d["count"], f"{name}: contact count at step {k}"
                assert hashlib.sha256(table.astype("<i4").tobytes()).hexdigest() == d["sha256"], \
                    f"{name}: contact table (ids, pairs, colors, feature ids) at step {k}"
