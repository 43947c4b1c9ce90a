"""Mixed-radix digits to binary on the device (and the host fallback for gcds with more
than 4,096 digits), and the exhaustive certification of the inverse's quotient steps."""
import math
import random

import pytest

pytestmark = pytest.mark.gpu


def test_device_conversion_around_the_digit_limit(mgcd):
    rng = random.Random(51)
    us, vs = [], []
    # gcd sizes from one limb to past the 4,096-digit device limit (32-bit moduli: about
    # 32 bits per digit); cofactors of 3,000 bits
    for gbits in (1, 31, 64, 1000, 32 * 2000, 32 * 4000, 32 * 4090, 32 * 4200, 200000):
        g = rng.getrandbits(gbits) | (1 << (gbits - 1)) | 1
        for _ in range(2):
            us.append(g * (rng.getrandbits(3000) | 1))
            vs.append(g * (rng.getrandbits(2900) | 1))
    with mgcd.Device(0, 32) as dev:
        assert dev.gcd_batch(us, vs) == [math.gcd(u, v) for u, v in zip(us, vs)]
        _, d2h = dev.batch_transfer_bytes()
        # results come back as limbs; digits only for the pairs past the device limit
        digit_bytes = sum(8 * (mgcd.moduli_needed(max(u, v).bit_length()) + 1) for u, v in zip(us, vs))
        assert d2h < digit_bytes


def test_single_pair_digits_and_value_agree(mgcd, oracle):
    rng = random.Random(52)
    with mgcd.Device(0, 32) as dev:
        for gbits in (2, 500, 20000):
            g = rng.getrandbits(gbits) | (1 << (gbits - 1))
            u, v = g * (rng.getrandbits(5000) | 1), g * (rng.getrandbits(4000) | 1)
            dig = dev.gcd_digits(u, v)
            val = dig[-1][1]
            for m, d in reversed(dig[:-1]):
                val = val * m + d
            assert abs(val) == math.gcd(u, v) == dev.gcd(u, v)


def test_inverse_quotient_steps_certified(mgcd):
    with mgcd.Device(0, 32) as dev:
        r = dev.certify_inverse()
    assert r["failures"] == 0, r
    assert r["checked"] > 5 * 10**10
