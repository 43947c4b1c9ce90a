"""Moduli grown on demand in batches (mgcd_set_growth): a pair starts with part of the
reference's moduli count and takes more from the table when its loop runs out of moduli or
ends uncertified.  Every gcd is compared with Python's exact gcd, and each pair's digits and
final moduli count with the oracle's restatement of the same policy (orc_modgcd_grow); a
pair the GPU could not certify at its cap was rerun with the reference's count, so its
digits are the reference loop's (orc_modgcd)."""
import importlib
import math
import random

import pytest

pytestmark = pytest.mark.gpu

wl = importlib.import_module("modgcd-onegpu_gb300.workloads")


def _check_against_oracle(dev, oracle, us, vs, L, start, permille):
    mods = oracle.gen_moduli(L, 20000)
    grown = 0
    for i, (u, v) in enumerate(zip(us, vs)):
        a, b = (u, v) if u >= v else (v, u)
        dig, nqf = dev.batch_pair_digits(i)
        ref = oracle.num_moduli_needed(a.bit_length(), L)
        n0 = oracle.grow_start_count(ref, start)
        st, odig, _, onf = oracle.modgcd_grow(a, b, L, mods, n0, oracle.grow_cap(ref), permille)
        if st != 0:                  # rerun by the host with the reference's count
            st, odig, _, _ = oracle.modgcd(a, b, L, mods, ref)
            onf = ref
        assert st == 0
        assert dig == odig, "pair %d (%d bits): digits differ" % (i, a.bit_length())
        assert nqf == onf
        grown += nqf > n0
    return grown


@pytest.mark.parametrize("L,start,permille", [(27, 0.4, 50), (32, 0.5, 50), (27, 0.2, 20)])
def test_growth_digits_match_oracle(mgcd, oracle, L, start, permille):
    us, vs, _ = wl.mixed_batch(160, seed=21, hi_bits=12000)
    with mgcd.Device(0, L) as dev:
        dev.set_growth(start, permille)
        assert dev.growth() == (pytest.approx(start), permille)
        res = dev.gcd_batch(us, vs)
        assert res == [math.gcd(u, v) for u, v in zip(us, vs)]
        grown = _check_against_oracle(dev, oracle, us, vs, L, start, permille)
    assert grown > 0                 # the policy was exercised


def test_growth_large_pairs_and_graph_replay(mgcd):
    """Class-2 pairs (up to 64k bits) with growth, run directly and replayed from a CUDA
    graph: identical exact results."""
    rng = random.Random(77)
    us, vs, _ = wl.mixed_batch(96, seed=23, lo_bits=20000, hi_bits=65536)
    for _ in range(8):               # v | u and coprime pairs stress the certification
        v = rng.getrandbits(rng.randint(20000, 40000)) | 1
        us.append(v * (rng.getrandbits(rng.randint(1, 64)) | 1))
        vs.append(v)
    exp = [math.gcd(u, v) for u, v in zip(us, vs)]
    with mgcd.Device(0, 27) as dev:
        dev.set_growth(0.5, 50)
        dev.batch_use_graph(True)
        dev.batch_upload(*mgcd.pack_pairs(us, vs))
        for _ in range(2):
            dev.batch_run()
            dev.batch_sync()
            g, g_off, g_len, st = dev.batch_download()
            assert (st == 0).all()
            assert [mgcd.from_limbs(g[int(o): int(o) + int(n)]) for o, n in zip(g_off, g_len)] == exp
        dev.batch_use_graph(False)


def test_growth_settings_validated(mgcd, tmp_path):
    with mgcd.Device(0, 32) as dev:
        for bad in [(0.05, 50), (1.5, 50), (0.5, 5), (0.5, 600)]:
            with pytest.raises(mgcd.GcdError):
                dev.set_growth(*bad)
        dev.set_growth(0.4, 80)
        path = str(tmp_path / "t.txt")
        dev.save_tuning(path)
        dev.set_growth(0)
        assert dev.growth()[0] == 0
        dev.load_tuning(path)
        assert dev.growth() == (pytest.approx(0.4), 80)
        bad = tmp_path / "bad.txt"
        bad.write_text("0 256 4 1.0 0\ngrow 0.05 50\n")
        with pytest.raises(mgcd.GcdError):
            dev.load_tuning(str(bad))
        assert dev.growth() == (pytest.approx(0.4), 80)       # nothing applied
