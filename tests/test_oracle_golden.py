"""The oracle and the generator reproduce the committed fixtures (tests/golden/oracle_fixtures.json,
made by tests/golden/make_golden.py): same scene bytes on every host, same frame digests."""
import json
from pathlib import Path

import pytest

import oracle
import webgs

FIXTURES = json.loads((Path(__file__).parent / "golden" / "oracle_fixtures.json").read_text())


@pytest.mark.parametrize("case", FIXTURES, ids=[c["name"] for c in FIXTURES])
def test_oracle_matches_fixture(case):
    import importlib.util

    spec = importlib.util.spec_from_file_location("make_golden", Path(__file__).parent / "golden" / "make_golden.py")
    mg = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mg)
    kind, count, seed, clusters, box = case["scene"]
    packed = webgs.synth_scene(kind, count, seed, clusters, box)
    assert mg.digest(packed) == case["scene_digest"], "generator output changed"
    vb = bytes.fromhex(case["view_hex"])
    r = oracle.forward_f32(vb, packed, count, tile=case["tile"], factor=case["factor"])
    got = mg.summarize(r)
    for key in ("instance_count", "sorted_count", "keys", "vals", "ranges", "rgb", "rgba8"):
        assert got[key] == case[key], key
