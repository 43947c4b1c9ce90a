"""The benchmark workloads' generator (no GPU): GMP's Mersenne Twister through libgmp.so.10.

Pinned against the reference itself: `reference_pairs` must reproduce, draw for draw, the
test-vector files the reference's own driver wrote (testmodgcd.cpp:219-229, default seed;
tests/golden/ref_*.txt).  The single-pair configuration's seed-1 pair is pinned by a
fixture, and the mixed batch keeps its stated shape."""
import importlib
import math

import pytest

from conftest import golden_pairs, parse_b62, GOLDEN

wl = importlib.import_module("modgcd-onegpu_gb300.workloads")


@pytest.mark.parametrize("case_idx", range(8))
def test_reference_stream_reproduced(golden, case_idx):
    case = golden["cases"][case_idx]
    pairs = golden_pairs(case)
    assert wl.reference_pairs(case["bits"], case["gcd_bits"], len(pairs)) == pairs


def test_single_pair_seed1_fixture():
    lines = [ln for ln in open(GOLDEN + "/config1_seed1.txt").read().split("\n") if ln.strip()]
    u, v, g = (parse_b62(x) for x in lines)
    assert wl.single_pair(seed=1) == (u, v)
    assert 10239 <= u.bit_length() <= 10240 and 10239 <= v.bit_length() <= 10240
    assert math.gcd(u, v) == g and g.bit_length() == 2048 and g & 1


def test_mixed_batch_shape():
    us, vs, kinds = wl.mixed_batch(400, seed=3)
    assert wl.mixed_batch(400, seed=3)[0] == us                  # deterministic
    assert wl.mixed_batch(400, seed=4)[0] != us
    for u, v, k in zip(us, vs, kinds):
        bu, bv = u.bit_length(), v.bit_length()
        assert 1000 <= bu <= 65536 + 1
        assert bv <= bu + 1 and 2 * bv >= bu - 2
        if k == "coprime":
            assert math.gcd(u, v) == 1
        elif k == "divides":
            assert u % v == 0
    frac = {k: kinds.count(k) / len(kinds) for k in ("coprime", "divides", "planted")}
    assert 0.18 < frac["coprime"] < 0.32 and frac["divides"] < 0.10 and 0.6 < frac["planted"] < 0.8


def test_sweep_and_serve_shapes():
    for n in (4096, 65536):
        u, v = wl.size_sweep_pair(n, seed=1)
        assert n - 1 <= u.bit_length() <= n and n - 1 <= v.bit_length() <= n
        assert math.gcd(u, v).bit_length() >= n // 4
    us, vs, arr = wl.serve_requests(300, 1000.0, seed=5)
    assert all(b > a for a, b in zip(arr, arr[1:]))
    assert sum(max(u.bit_length(), v.bit_length()) > (1 << 19) for u, v in zip(us, vs)) == 3
