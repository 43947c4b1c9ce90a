"""Failure detection on the GPU without faulting it.

- A bounded wait that runs out: one CTA of a cooperative-grid pair withholds its
  publication (a flag nothing sets); the other CTAs give up after the bound, the pair fails
  with MGCD_ERR_TIMEOUT, and the same context then computes correctly.
- Operand staging that fails (host-set hook, reported after the bulk copies completed):
  every CTA of an affected pair stops at the first exchange -- on one CTA, a cluster and the
  cooperative grid -- the pair fails with MGCD_ERR_TIMEOUT, the other pairs of a batch are
  exact, and the context then computes correctly.
- Too few moduli (host-side injection): every pair is forced onto a moduli count that cannot
  hold it.  The reference's own check (sizes tracked with __ffs) misses such cases and its
  kernel can return a wrong gcd; here the result is certified on the device, so the call
  must fail with the reference's "ran out of moduli" error instead.
"""
import math
import random

import pytest

pytestmark = pytest.mark.gpu


def _pair(rng, nbits, gbits):
    g = rng.getrandbits(gbits) | (1 << (gbits - 1))
    return g * (rng.getrandbits(nbits - gbits) | 1), g * (rng.getrandbits(nbits - gbits) | 1)


@pytest.mark.parametrize("policy", [0, 2])
def test_grid_wait_runs_out_and_context_survives(mgcd, policy):
    """policy 0: CTA 1 of the cooperative grid withholds; policy 2: cluster 1 of the grid
    of clusters does."""
    rng = random.Random(31)
    u, v = _pair(rng, 420000, 60000)          # > 16,384 moduli: cooperative grid
    with mgcd.Device(0, 32) as dev:
        dev.set_single_pair_policy(policy)
        dev.set_wait_timeout_ms(200)
        dev.test_withhold_cta(1)
        with pytest.raises(mgcd.GcdError) as e:
            dev.gcd(u, v)
        assert mgcd.STATUS_NAMES[e.value.status] == "MGCD_ERR_TIMEOUT"
        dev.test_withhold_cta(-1)
        assert dev.gcd(u, v) == math.gcd(u, v)
        a, b = _pair(rng, 3000, 500)
        assert dev.gcd(a, b) == math.gcd(a, b)


@pytest.mark.parametrize("nbits,forced", [(65536, 4608), (65536, 5120), (20000, 1024)])
def test_too_few_moduli_never_returns_a_wrong_gcd(mgcd, nbits, forced):
    rng = random.Random(nbits + forced)
    u, v = _pair(rng, nbits, 8)
    with mgcd.Device(0, 32) as dev:
        dev.test_force_moduli(forced)
        try:
            g = dev.gcd(u, v)
        except mgcd.GcdError as e:
            assert str(e) in ("Ran out of moduli in the reduction loop.",
                              "Ran out of moduli in the recovery loop.")
        else:
            assert g == math.gcd(u, v)
        res, st = dev.gcd_batch([u, u + 2, v], [v, v, u + 6], return_status=True)
        for r, s, (a, b) in zip(res, st, [(u, v), (u + 2, v), (v, u + 6)]):
            assert s in (0, 6, 7)
            if s == 0:
                assert r == math.gcd(a, b)
        dev.test_force_moduli(0)
        assert dev.gcd(u, v) == math.gcd(u, v)


def test_staging_failure_stops_pair_and_context_survives(mgcd):
    rng = random.Random(32)
    small = [_pair(rng, nb, nb // 4) for nb in (2000, 3000, 9000, 30000) for _ in range(40)]
    big = [_pair(rng, 300000, 40000) for _ in range(2)]            # size class 3: clusters
    cluster_pair = _pair(rng, 60000, 9000)                          # single pair, cluster
    grid_pair = _pair(rng, 420000, 60000)                           # single pair, grid
    with mgcd.Device(0, 32) as dev:
        dev.set_wait_timeout_ms(200)
        dev.test_fail_staging(1)
        for u, v in (cluster_pair, grid_pair):
            with pytest.raises(mgcd.GcdError) as e:
                dev.gcd(u, v)
            assert mgcd.STATUS_NAMES[e.value.status] == "MGCD_ERR_TIMEOUT"
        us = [u for u, _ in small + big]
        vs = [v for _, v in small + big]
        res, st = dev.gcd_batch(us, vs, return_status=True)
        names = {mgcd.STATUS_NAMES[int(x)] for x in st}
        assert names <= {"MGCD_OK", "MGCD_ERR_TIMEOUT"}
        assert "MGCD_ERR_TIMEOUT" in names                       # CTA 1 took some pairs
        for (u, v), r, x in zip(small + big, res, st):
            if mgcd.STATUS_NAMES[int(x)] == "MGCD_OK":
                assert r == math.gcd(u, v)
        dev.test_fail_staging(-1)
        for u, v in (cluster_pair, grid_pair):
            assert dev.gcd(u, v) == math.gcd(u, v)
        assert dev.gcd_batch(us, vs) == [math.gcd(u, v) for u, v in zip(us, vs)]
