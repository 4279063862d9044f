"""The oracle reproduces the committed golden digests (tests/golden/golden.json)
for the benchmark configurations at full size and two small cases: the
fixtures the GPU parity tests compare against stay the oracle's output."""
import pytest

from tests.golden import make_golden


@pytest.mark.parametrize("name", list(make_golden.CASES))
def test_oracle_matches_golden(name):
    want = make_golden.load()["cases"][name]
    got = make_golden.oracle_values(name)
    for key, value in got.items():
        assert want[key] == value, key
