"""CPU: the oracle reproduces its committed regression fixtures (tests/golden/oracle_fixtures.json, made
by tests/golden/make_fixtures.py).  The fixtures pin the restatement against unintended changes; they
are not reference outputs."""

import json
from pathlib import Path

import pytest

from tests.golden import make_fixtures

FIXTURES = json.loads((Path(__file__).resolve().parent / "golden" / "oracle_fixtures.json").read_text())


@pytest.mark.parametrize("want", FIXTURES, ids=[f"{f['splats']}-{f['seed']}" for f in FIXTURES])
def test_oracle_reproduces_its_fixtures(oracle, want):
    got = make_fixtures.fixture(oracle, want["splats"], want["seed"], want["layout"], tuple(want["eye"]),
                                want["width"], want["height"])
    for k in ("visible", "keys_sha256", "index_sha256", "fragments"):
        assert got[k] == want[k], k
    assert got["image_sum"] == pytest.approx(want["image_sum"], rel=1e-12)
    assert got["image_center"] == pytest.approx(want["image_center"], rel=1e-12, abs=1e-12)
