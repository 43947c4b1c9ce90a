"""GPU parity: the CUDA path against the oracle, bit for bit.

Final results against GMP mpz_gcd / Python's exact gcd; the digit list (the kernel's
pair_t output) against the restated reference algorithm, element by element."""
import hashlib
import math
import os
import random
import subprocess

import numpy as np
import pytest

from conftest import GOLDEN, golden_pairs

pytestmark = pytest.mark.gpu


def rand_pair(rng, nbits, gbits, vbits=None):
    g = rng.getrandbits(gbits) | (1 << (gbits - 1)) if gbits > 0 else 1
    a = rng.getrandbits(max(nbits - gbits, 1)) | 1
    b = rng.getrandbits(max((vbits or nbits) - gbits, 1)) | 1
    return g * a, g * b


@pytest.mark.parametrize("case_idx", range(8))
def test_golden_reference_inputs(device, golden, case_idx):
    """The reference driver's own inputs: gcd exact, digits identical to the oracle's."""
    case = golden["cases"][case_idx]
    pairs = golden_pairs(case)
    for (u, v), exp in zip(pairs, case["pairs"]):
        g = int(exp["gcd_hex"], 16)
        assert device.gcd(u, v) == g
        dig = device.gcd_digits(u, v)
        assert len(dig) == exp["digits"]
        assert hashlib.sha1(repr(dig).encode()).hexdigest() == exp["digits_sha1"]
    res = device.gcd_batch([u for u, _ in pairs], [v for _, v in pairs])
    assert res == [int(e["gcd_hex"], 16) for e in case["pairs"]]


def test_digits_match_oracle_random(device, oracle):
    rng = random.Random(11)
    mod32 = oracle.gen_moduli(32, 4096)
    for nbits, gbits in [(64, 1), (300, 50), (1000, 1), (2048, 700), (4096, 1024), (8000, 4000)]:
        for _ in range(3):
            u, v = rand_pair(rng, nbits, gbits)
            uu, vv = max(u, v), min(u, v)
            nq = oracle.num_moduli_needed(uu.bit_length(), 32)
            st, dig, tr, it = oracle.modgcd(uu, vv, 32, mod32, nq)
            assert st == 0
            assert device.gcd_digits(u, v) == dig
            assert device.gcd(u, v) == math.gcd(u, v)


def test_batch_mixed_sizes(device):
    rng = random.Random(12)
    us, vs = [], []
    for _ in range(300):
        nb = int(2 ** rng.uniform(6, 14.5))
        gb = rng.randint(0, nb // 2)
        u, v = rand_pair(rng, nb, gb, vbits=max(gb + 1, int(nb / rng.uniform(1, 2))))
        us.append(u)
        vs.append(v)
    res = device.gcd_batch(us, vs)
    assert res == [math.gcd(u, v) for u, v in zip(us, vs)]


@pytest.mark.parametrize("scale", [0.8, 0.5])
def test_batch_fewer_moduli_certified(mgcd, scale):
    """Batches with fewer moduli than the reference count: every result certified or rerun
    with the reference count -- results stay exact.  At 0.5 many pairs need the rerun."""
    wl = __import__("importlib").import_module("modgcd-onegpu_gb300.workloads")
    us, vs, _ = wl.mixed_batch(200, seed=9, hi_bits=20000)
    with mgcd.Device(0, 32) as dev:
        dev.set_growth(0)            # fixed counts: the rerun path
        dev.set_nq_scale(scale)
        res = dev.gcd_batch(us, vs)
        retried = dev.batch_retried()
    assert res == [math.gcd(u, v) for u, v in zip(us, vs)]
    if scale == 0.5:
        assert retried > 0


def test_edge_cases(device):
    rng = random.Random(13)
    x = rng.getrandbits(5000) | 1
    q0 = 4294967291
    cases = [(x, x), (x * 987654321, x), (x, x * 3), (x << 64, x), (1, 1), (1, 2), (2, 1),
             (0xFFFFFFFF, 0xFFFFFFFB), (2 ** 32, 2 ** 31), (q0 * x, q0 * 7), (q0 ** 3, q0 ** 2 * 5),
             (x, 0), (0, x), (0, 0), (2 ** 4000, 2 ** 3999 * 3)]
    for u, v in cases:
        assert device.gcd(u, v) == math.gcd(u, v), (u.bit_length(), v.bit_length())
    res = device.gcd_batch([u for u, _ in cases], [v for _, v in cases])
    assert res == [math.gcd(u, v) for u, v in cases]


def test_order_and_leading_zero_limbs(device, mgcd):
    rng = random.Random(14)
    u, v = rand_pair(rng, 3000, 500)
    a, b = mgcd.to_limbs(u), mgcd.to_limbs(v)
    z = np.zeros(2, dtype=np.uint32)
    # pair 0: (v, u) with two zero limbs above v's top limb; pair 1: (u, v) sharing the limbs
    limbs = np.concatenate([b, z, a]).astype(np.uint32)
    uo = np.array([0, len(b) + 2], dtype=np.uint64)
    ul = np.array([len(b) + 2, len(a)], dtype=np.uint32)
    vo = np.array([len(b) + 2, 0], dtype=np.uint64)
    vl = np.array([len(a), len(b)], dtype=np.uint32)
    g, g_off, g_len, st = device.gcd_batch_packed(limbs, uo, ul, vo, vl)
    assert list(st) == [0, 0]
    for i in range(2):
        assert mgcd.from_limbs(g[int(g_off[i]): int(g_off[i]) + int(g_len[i])]) == math.gcd(u, v)


def test_batch_result_layouts(device, mgcd):
    """mgcd_gcd_batch with the caller's result slots: contiguous slots after a 3-limb margin
    (results copied back in place; nothing outside the slots touched), slots with 5-limb
    gaps (the compact layout; the gaps keep their contents), and contiguous slots of which
    one is a limb short of its gcd (that pair alone fails with the capacity error)."""
    rng = random.Random(29)
    us, vs = [], []
    for nbits, gbits in [(100, 40), (3000, 700), (20000, 5000), (64, 1), (9000, 2000), (40000, 9000)]:
        u, v = rand_pair(rng, nbits, gbits)
        us.append(u)
        vs.append(v)
    us.append(0)
    vs.append(123456789)                       # decided on the host
    exp = [math.gcd(u, v) for u, v in zip(us, vs)]
    n = len(us)
    limbs, uo, ul, vo, vl = mgcd.pack_pairs(us, vs)
    off, cap, tot = mgcd.result_layout(ul, vl)
    SENT = 0xA5A5A5A5

    def run(off, cap, size):
        g = np.full(size, SENT, dtype=np.uint32)
        gl = np.zeros(n, dtype=np.uint32)
        st = np.zeros(n, dtype=np.int32)
        device.gcd_batch_packed(limbs, uo, ul, vo, vl, out=(g, off, cap, gl, st))
        res = [mgcd.from_limbs(g[int(o): int(o) + int(k)]) for o, k in zip(off, gl)]
        return g, gl, st, res

    off1 = off + np.uint64(3)
    g, gl, st, res = run(off1, cap, tot + 7)
    assert list(st) == [0] * n and res == exp
    assert (g[:3] == SENT).all() and (g[tot + 3:] == SENT).all()

    off2 = off + np.uint64(5) * np.arange(n, dtype=np.uint64)
    g, gl, st, res = run(off2, cap, tot + 5 * n)
    assert list(st) == [0] * n and res == exp
    for i in range(n):
        end = int(off2[i]) + int(cap[i])
        assert (g[end: end + 5] == SENT).all()

    k = 2
    need = (exp[k].bit_length() + 31) // 32
    cap3 = cap.copy()
    cap3[k] = need - 1
    off3 = np.zeros(n, dtype=np.uint64)
    off3[1:] = np.cumsum(cap3[:-1], dtype=np.uint64)
    g, gl, st, res = run(off3, cap3, int(cap3.sum(dtype=np.uint64)))
    assert st[k] == mgcd.MGCD_ERR_CAPACITY and gl[k] == 0
    assert [int(s) for i, s in enumerate(st) if i != k] == [0] * (n - 1)
    assert [r for i, r in enumerate(res) if i != k] == [e for i, e in enumerate(exp) if i != k]


@pytest.mark.parametrize("L", [22, 27])
def test_other_modulus_widths(mgcd, oracle, L):
    rng = random.Random(15 + L)
    with mgcd.Device(0, L) as dev:
        mods = oracle.gen_moduli(L, 8192)
        us, vs = [], []
        for nbits, gbits in [(100, 1), (1000, 300), (4096, 1024), (10000, 2500)]:
            u, v = rand_pair(rng, nbits, gbits)
            uu, vv = max(u, v), min(u, v)
            nq = oracle.num_moduli_needed(uu.bit_length(), L)
            st, dig, _, _ = oracle.modgcd(uu, vv, L, mods, nq)
            assert st == 0
            assert dev.gcd_digits(u, v) == dig
            us.append(u)
            vs.append(v)
        assert dev.gcd_batch(us, vs) == [math.gcd(a, b) for a, b in zip(us, vs)]


def test_large_pairs_clusters_and_grid(device):
    """Pairs too large for one CTA: single pairs on a cluster (up to 8,192 moduli) or the
    cooperative grid; in a batch, on clusters from the size-class-3 queue."""
    rng = random.Random(16)
    u, v = rand_pair(rng, 65536, 16384)
    assert device.gcd(u, v) == math.gcd(u, v)                       # plain, cluster
    u3, v3 = rand_pair(rng, 420000, 100000)
    assert device.gcd(u3, v3) == math.gcd(u3, v3)                   # plain, grid
    u2, v2 = rand_pair(rng, 262144, 65536)
    assert device.gcd_batch([u2, u], [v2, v]) == [math.gcd(u2, v2), math.gcd(u, v)]


def test_single_pair_launch_shapes_agree(mgcd, oracle):
    """Cluster (DSMEM exchange), cooperative grid and the reference's launch shape give
    the oracle's digits."""
    rng = random.Random(17)
    mod32 = oracle.gen_moduli(32, 8192)
    with mgcd.Device(0, 32) as dev:
        for nbits, gbits in [(3000, 700), (20000, 5000), (60000, 15000)]:
            u, v = rand_pair(rng, nbits, gbits)
            uu, vv = max(u, v), min(u, v)
            nq = oracle.num_moduli_needed(uu.bit_length(), 32)
            st, dig, _, _ = oracle.modgcd(uu, vv, 32, mod32, nq)
            assert st == 0
            dev.set_single_pair_policy(0)
            assert dev.gcd_digits(u, v) == dig
            dev.set_single_pair_policy(1)
            assert dev.gcd_digits(u, v) == dig
        # 26,880 and 34,816 moduli: the cooperative grid, the reference's shape, the grid of
        # 8-CTA clusters (digits compared with the oracle's at the smaller size)
        for nbits in (300000, 400000):
            u, v = rand_pair(rng, nbits, 80000)
            g = math.gcd(u, v)
            for pol in (0, 1, 2):
                dev.set_single_pair_policy(pol)
                assert dev.gcd(u, v) == g
        uu, vv = max(u, v), min(u, v)
        nq = oracle.num_moduli_needed(uu.bit_length(), 32)
        st, dig, _, _ = oracle.modgcd(uu, vv, 32, oracle.gen_moduli(32, nq), nq)
        assert st == 0
        dev.set_single_pair_policy(2)
        assert dev.gcd_digits(u, v) == dig


def test_not_enough_moduli(mgcd):
    with mgcd.Device(0, 22) as dev:
        x = (1 << 1_300_000) + 1
        with pytest.raises(mgcd.GcdError) as e:
            dev.gcd(x, x - 2)
        assert str(e.value) == "Not enough moduli available for given input."


def test_cpp_dropin_driver(mgcd):
    exe = os.path.join(mgcd.LIB_DIR, "testmodgcd_gb300")
    for f in ("ref_1024-1.txt", "ref_10240-2048.txt", "ref_16384-4096.txt"):
        for extra in ([], ["--batch"]):
            r = subprocess.run([exe, "file", os.path.join(GOLDEN, f)] + extra, capture_output=True, text=True)
            assert r.returncode == 0, r.stdout + r.stderr
            assert '"mismatches": 0, "errors": 0' in r.stdout
    r = subprocess.run([exe, "rand", "5000", "1200", "6", "42"], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr


def test_operand_staging_alignment_and_tile_edges(mgcd, device):
    """Operand tiles reach shared memory by bulk copies widened to 16-byte bounds: every
    operand start modulo 4 limbs and lengths around the 1,024-limb tile edge, in the batched
    kernels, on a cluster and on the cooperative grid, against Python's gcd."""
    rng = random.Random(23)
    us, vs = [], []
    for ulimbs in (1, 3, 4, 5, 1023, 1024, 1025, 2049):
        for gl in (0, 1):
            u, v = rand_pair(rng, 32 * ulimbs, 16 * ulimbs * gl, max(2, 32 * ulimbs - 5))
            us.append(u)
            vs.append(v)
    for shift in range(4):
        # a gap of `shift` limbs before every operand moves its start through all four
        # positions inside a 16-byte line
        parts, uo, ul, vo, vl = [np.zeros(shift, dtype=np.uint32)], [], [], [], []
        off = shift
        for u, v in zip(us, vs):
            a, b = mgcd.to_limbs(u), mgcd.to_limbs(v)
            uo.append(off); ul.append(len(a)); parts.append(a); off += len(a)
            parts.append(np.zeros(shift, dtype=np.uint32)); off += shift
            vo.append(off); vl.append(len(b)); parts.append(b); off += len(b)
            parts.append(np.zeros(shift, dtype=np.uint32)); off += shift
        packed = (np.ascontiguousarray(np.concatenate(parts), dtype=np.uint32), np.array(uo, dtype=np.uint64),
                  np.array(ul, dtype=np.uint32), np.array(vo, dtype=np.uint64), np.array(vl, dtype=np.uint32))
        g, g_off, g_len, st = device.gcd_batch_packed(*packed)
        assert (st == 0).all()
        for i, (u, v) in enumerate(zip(us, vs)):
            o = int(g_off[i])
            assert mgcd.from_limbs(g[o:o + int(g_len[i])]) == math.gcd(u, v), (shift, i)
    # single pairs: 1025 limbs on a cluster, 9000 limbs (~33,000 moduli) on the grid
    for nl in (1025, 9000):
        u, v = rand_pair(rng, 32 * nl, 8 * nl)
        assert device.gcd(u, v) == math.gcd(u, v)


def test_one_megabit_pair_at_22bit_moduli(mgcd, oracle):
    """The single-pair sweep's largest case at full size: 1M-bit operands with a 256k-bit
    planted gcd, 22-bit moduli (96,256 of them), against GMP mpz_gcd."""
    wl = __import__("importlib").import_module("modgcd-onegpu_gb300.workloads")
    u, v = wl.size_sweep_pair(1 << 20, seed=1)
    _, g, go, gn = oracle.cpu_gmp_gcd_batch(*mgcd.pack_pairs([u], [v]), 1)
    expect = oracle.from_limbs(g[: int(gn[0])])
    assert expect.bit_length() >= 1 << 18
    with mgcd.Device(0, 22) as dev:
        assert dev.gcd(u, v) == expect
