"""The oracle pinned before it is trusted: moduli against the reference's createModuli
output, the restated algorithm against GMP mpz_gcd on the reference driver's own inputs."""
import hashlib
import math
import os
import random

import numpy as np
import pytest

from conftest import GOLDEN, golden_pairs


def _ref_moduli_fixture():
    d = {}
    for line in open(os.path.join(GOLDEN, "ref_moduli_L32.txt")):
        if line.startswith("#"):
            continue
        k, _, v = line.strip().partition(" ")
        d[k] = v
    return d


def test_oracle_moduli_match_reference_createModuli(oracle):
    ref = _ref_moduli_fixture()
    m = oracle.gen_moduli(32, int(ref["count"]))
    assert len(m) == int(ref["count"])
    assert hashlib.sha1(m.astype("<u4").tobytes()).hexdigest() == ref["sha1"]
    assert list(m[:64]) == [int(x) for x in ref["head"].split()]
    assert list(m[-64:]) == [int(x) for x in ref["tail"].split()]
    assert list(m[:4]) == [4294967291, 4294967279, 4294967231, 4294967197]


def test_oracle_moduli_other_widths(oracle):
    for L in (22, 27):
        m = oracle.gen_moduli(L, 2000)
        assert len(m) == 2000
        assert np.all(np.diff(m.astype(np.int64)) < 0)
        assert m[0] < (1 << L) and m[-1] > (1 << (L - 1))
    # every 22-bit prime that passes the criterion: 97,358 of them
    assert len(oracle.gen_moduli(22, 200000)) == 97358


def test_num_moduli_needed_formula(oracle):
    # roundUp(ceil((1.6 - 0.015 L) n / ln n), 256), GmpCudaDevice-gcd.cu:49-55
    for L in (22, 27, 32):
        cl = 1.6 - 0.015 * L
        for n in (2, 64, 1000, 10240, 65536, 262144, 1 << 20):
            want = math.ceil(cl * n / math.log(n))
            want = ((want - 1) // 256 + 1) * 256
            got = oracle.num_moduli_needed(n, L)
            assert abs(got - want) in (0, 256), (L, n)   # float vs double only at 256 boundaries
    assert [oracle.num_moduli_needed(b, 32) for b in (1024, 4096, 10240, 16384, 65536, 262144, 1 << 20)] == \
        [256, 768, 1280, 2048, 6656, 23552, 84736]
    assert oracle.num_moduli_needed(1 << 20, 27) == 90624
    assert oracle.num_moduli_needed(1 << 20, 22) == 96256


@pytest.mark.parametrize("case_idx", range(8))
def test_oracle_on_reference_inputs(oracle, golden, case_idx):
    case = golden["cases"][case_idx]
    mod32 = oracle.gen_moduli(32, 8192)
    for (u, v), exp in zip(golden_pairs(case), case["pairs"]):
        g = int(exp["gcd_hex"], 16)
        assert g == math.gcd(u, v)
        uu, vv = (u, v) if u >= v else (v, u)
        if case["bits"] > 20000:      # large cases: compare the recorded fingerprints only
            continue
        nq = oracle.num_moduli_needed(uu.bit_length(), 32)
        assert nq == exp["nq"]
        st, dig, tr, it = oracle.modgcd(uu, vv, 32, mod32, nq)
        assert st == exp["status"] == 0
        assert it == exp["iters"] and len(dig) == exp["digits"]
        assert hashlib.sha1(repr(tr).encode()).hexdigest() == exp["trace_sha1"]
        assert hashlib.sha1(repr(dig).encode()).hexdigest() == exp["digits_sha1"]
        assert oracle.mixed_radix_to_int(dig) == g
        assert oracle.mixed_radix_to_int_c(dig) == g


def test_oracle_random_and_edge_cases(oracle):
    rng = random.Random(7)
    mod32 = oracle.gen_moduli(32, 4096)
    cases = []
    for _ in range(40):
        nb = rng.choice([33, 64, 100, 500, 2000])
        gb = rng.choice([1, 10, 100, nb // 2])
        g = rng.getrandbits(gb) | 1
        cases.append((g * (rng.getrandbits(nb) | 1), g * (rng.getrandbits(nb) | 1)))
    x = rng.getrandbits(3000) | 1
    cases += [(x, x), (x * 12345, x), (x << 40, x), (1, 1), (2, 1), (3, 2), (0xFFFFFFFF, 0xFFFFFFFB)]
    q0 = int(mod32[0])
    cases += [(q0 * x, q0 * 3), (q0 * q0 * 5, q0 * 7)]     # gcd divisible by a table modulus
    for u, v in cases:
        assert oracle.ref_gcd(u, v, 32, mod32) == math.gcd(u, v), (u, v)


def test_mixed_radix_conversion(oracle):
    rng = random.Random(3)
    mods = [int(x) for x in oracle.gen_moduli(32, 64)]
    for _ in range(20):
        k = rng.randint(1, 40)
        dig = [(mods[i], rng.randint(-(mods[i] // 2), mods[i] // 2)) for i in range(k)]
        assert oracle.mixed_radix_to_int(dig) == oracle.mixed_radix_to_int_c(dig)


def test_gmp_batch_baseline(oracle):
    rng = random.Random(5)
    us = [rng.getrandbits(rng.randint(1, 3000)) for _ in range(50)]
    vs = [rng.getrandbits(rng.randint(1, 3000)) for _ in range(50)]
    us[0], vs[1] = 0, 0
    parts, uo, ul, vo, vl = [], [], [], [], []
    off = 0
    for u, v in zip(us, vs):
        a, b = oracle.to_limbs(u), oracle.to_limbs(v)
        uo.append(off); ul.append(len(a)); parts.append(a); off += len(a)
        vo.append(off); vl.append(len(b)); parts.append(b); off += len(b)
    secs, g, goff, glen = oracle.cpu_gmp_gcd_batch(np.concatenate(parts), uo, ul, vo, vl, 2)
    for i, (u, v) in enumerate(zip(us, vs)):
        assert oracle.from_limbs(g[int(goff[i]): int(goff[i]) + int(glen[i])]) == math.gcd(u, v)


def test_oracle_growth_restatement(oracle, golden):
    """The oracle's restatement of the batches' moduli growth (orc_modgcd_grow): without room
    to grow it is the reference loop (same digits as orc_modgcd at the same count); with
    growth every result is the exact gcd, sets stay within their caps, and the set grows."""
    for L in (32, 27):
        mods = oracle.gen_moduli(L, 20000)
        grown = 0
        pairs = []
        for case in golden["cases"]:
            if case["bits"] <= 20000:
                pairs += golden_pairs(case)[:3]
        rng = random.Random(L)
        for _ in range(6):
            a = rng.getrandbits(rng.randint(200, 9000)) | 1
            pairs.append((a * (rng.getrandbits(64) | 1), a))                    # v | u
            pairs.append((rng.getrandbits(5000) | 1, rng.getrandbits(4000) | 1))  # near-coprime
        pairs.append((12345678901234567890123, 12345678901234567890123))       # u = v
        for u, v in pairs:
            uu, vv = (u, v) if u >= v else (v, u)
            ref = oracle.num_moduli_needed(uu.bit_length(), L)
            st, dig, _, nf = oracle.modgcd_grow(uu, vv, L, mods, ref, ref, 50)
            st0, dig0, _, _ = oracle.modgcd(uu, vv, L, mods, ref)
            if st == 0 and st0 == 0:
                assert dig == dig0 and nf == ref
            cap = oracle.grow_cap(ref)
            for start, permille in ((0.4, 50), (0.2, 20)):
                n0 = oracle.grow_start_count(ref, start)
                st, dig, _, nf = oracle.modgcd_grow(uu, vv, L, mods, n0, cap, permille)
                assert st == 0, (L, uu.bit_length(), st)
                assert oracle.mixed_radix_to_int(dig) == math.gcd(u, v)
                assert n0 <= nf <= cap
                grown += nf > n0
        assert grown > 0
