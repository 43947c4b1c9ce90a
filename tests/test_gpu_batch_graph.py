"""Batches holding pairs larger than one CTA (size class 3: one thread-block cluster per
pair, pulled from a persistent queue) and batches replayed from a recorded CUDA graph.
Every result is compared with Python's exact gcd; graph replays must equal direct runs."""
import importlib
import math
import os
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pair(rng, nbits, gbits):
    g = rng.getrandbits(gbits) | (1 << (gbits - 1)) if gbits > 0 else 1
    return (g * (rng.getrandbits(max(nbits - gbits, 1)) | 1),
            g * (rng.getrandbits(max(nbits - gbits, 1)) | 1))


def _skewed(rng, n_large, large_bits, n_small):
    """n_large pairs of large_bits bits plus n_small pairs of 512..4096 bits, random
    planted gcd sizes (the skewed-batch shape, scaled down)."""
    us, vs = [], []
    for _ in range(n_large):
        u, v = _pair(rng, large_bits, rng.randint(0, large_bits // 2))
        us.append(u)
        vs.append(v)
    for _ in range(n_small):
        nb = rng.randint(512, 4096)
        u, v = _pair(rng, nb, rng.randint(0, nb // 2))
        us.append(u)
        vs.append(v)
    return us, vs


def _results(mgcd, dev):
    g, g_off, g_len, st = dev.batch_download()
    assert (st == 0).all()
    return [mgcd.from_limbs(g[int(o): int(o) + int(n)]) for o, n in zip(g_off, g_len)]


def test_batch_with_cluster_class_pairs(mgcd):
    rng = random.Random(41)
    us, vs = _skewed(rng, 5, 300000, 200)
    with mgcd.Device(0, 32) as dev:
        assert dev.gcd_batch(us, vs) == [math.gcd(u, v) for u, v in zip(us, vs)]
        assert dev.get_cluster_size() == 8


@pytest.mark.parametrize("ctas", [2, 4, 16])
def test_cluster_sizes_agree(mgcd, ctas):
    rng = random.Random(42)
    us, vs = _skewed(rng, 3, 200000, 20)
    with mgcd.Device(0, 32) as dev:
        dev.set_cluster_size(ctas)
        assert dev.gcd_batch(us, vs) == [math.gcd(u, v) for u, v in zip(us, vs)]


def test_cluster_size_rejects_out_of_range(mgcd):
    with mgcd.Device(0, 32) as dev:
        for bad in (0, 1, 17):
            with pytest.raises(mgcd.GcdError):
                dev.set_cluster_size(bad)
        for bad in ((3, 1024, 8, 1.0), (0, 768, 1, 1.0), (1, 256, 3, 1.0), (2, 512, 2, 0.4)):
            with pytest.raises(mgcd.GcdError):
                dev.set_size_class(*bad)


def test_graph_replay_matches_direct(mgcd):
    rng = random.Random(43)
    us, vs = _skewed(rng, 2, 250000, 3000)
    exp = [math.gcd(u, v) for u, v in zip(us, vs)]
    packed = mgcd.pack_pairs(us, vs)
    with mgcd.Device(0, 32) as dev:
        dev.batch_upload(*packed)
        dev.batch_run()
        dev.batch_sync()
        direct_launches = dev.batch_launches()
        assert _results(mgcd, dev) == exp

        dev.batch_use_graph(True)
        for _ in range(3):
            dev.batch_run()
            dev.batch_sync()
            assert dev.batch_launches() == direct_launches
            assert _results(mgcd, dev) == exp

        # a new upload records a new graph; the old plan's buffers are not reused stale
        us2, vs2 = _skewed(random.Random(44), 1, 120000, 500)
        dev.batch_upload(*mgcd.pack_pairs(us2, vs2))
        dev.batch_run()
        dev.batch_sync()
        assert _results(mgcd, dev) == [math.gcd(u, v) for u, v in zip(us2, vs2)]
        dev.batch_use_graph(False)


def test_graph_replay_with_fewer_moduli_and_retries(mgcd):
    """Scaled moduli counts under graph replay: uncertified pairs are rerun outside the
    graph (direct launches) and the next replay still gives exact results."""
    rng = random.Random(45)
    us, vs = _skewed(rng, 0, 0, 1500)
    for _ in range(40):   # coprime-ish and v | u pairs push the certification bound
        nb = rng.randint(3000, 20000)
        v = rng.getrandbits(nb) | 1
        us.append(v * (rng.getrandbits(rng.randint(1, 64)) | 1))
        vs.append(v)
    exp = [math.gcd(u, v) for u, v in zip(us, vs)]
    with mgcd.Device(0, 32) as dev:
        dev.set_growth(0)            # fixed counts: the rerun path
        dev.set_nq_scale(0.5)
        dev.batch_use_graph(True)
        dev.batch_upload(*mgcd.pack_pairs(us, vs))
        for _ in range(2):
            dev.batch_run()
            dev.batch_sync()
            assert _results(mgcd, dev) == exp


def test_tuning_table_roundtrip_and_bad_tables(mgcd, tmp_path):
    with mgcd.Device(0, 32) as dev:
        dev.set_size_class(1, 256, 2, 0.9)
        dev.set_cluster_size(4)
        path = tmp_path / "table.txt"
        dev.save_tuning(str(path))
        dev.set_size_class(1, 512, 4, 1.0)
        dev.set_cluster_size(8)
        dev.load_tuning(str(path))
        t, k, s = dev.get_size_class(1)
        assert (t, k) == (256, 2) and abs(s - 0.9) < 1e-6
        assert dev.get_cluster_size() == 4
        before = [dev.get_size_class(c) for c in range(4)]
        for bad in ("1 256 2 0.9 0\n2 256 8 1.0 0\n",       # k = 8 needs 512 or 1024 threads
                    "3 1024 1 1.0 0\n",                       # class 3 needs a cluster size
                    "0 256 4 0.4 0\n",                        # scale below 0.5
                    "0 256 4\n"):                             # short line
            p = tmp_path / "bad.txt"
            p.write_text(bad)
            with pytest.raises(mgcd.GcdError):
                dev.load_tuning(str(p))
            assert [dev.get_size_class(c) for c in range(4)] == before   # nothing applied
        default = mgcd.default_tuning_path(dev)
        if os.path.exists(default):
            dev.load_tuning(default)
            rng = random.Random(46)
            us, vs = _skewed(rng, 1, 200000, 300)
            assert dev.gcd_batch(us, vs) == [math.gcd(u, v) for u, v in zip(us, vs)]


@pytest.mark.parametrize("threads,k,ctas,scale", [(512, 2, 8, 1.0), (512, 4, 16, 1.0), (256, 4, 8, 1.0),
                                                  (512, 2, 4, 0.6)])
def test_cluster_class_k_pairs_per_cluster(mgcd, threads, k, ctas, scale):
    """Class-3 pairs k to a cluster in lockstep (shared inverses); slots refill from the
    queue; with a low moduli fraction some pairs fail certification and are rerun."""
    rng = random.Random(48 + 3 * k + ctas)
    us, vs = _skewed(rng, 5, 230000, 40)
    v = rng.getrandbits(120000) | 1                 # v | u
    us.append(v * (rng.getrandbits(100000) | 1))
    vs.append(v)
    us.append(rng.getrandbits(240000) | 1)          # (almost surely) coprime
    vs.append(rng.getrandbits(239000) | 1)
    with mgcd.Device(0, 32) as dev:
        dev.set_size_class(3, threads, k, scale)
        dev.set_cluster_size(ctas)
        assert dev.gcd_batch(us, vs) == [math.gcd(a, b) for a, b in zip(us, vs)]


@pytest.mark.parametrize("threads,k", [(512, 4), (512, 8), (1024, 4), (1024, 8)])
def test_pairs_per_cta_step_down_when_shared_memory_is_short(mgcd, threads, k):
    """A size-class-2 pair near 16,384 moduli with k pairs per CTA would need more than one
    CTA's shared memory; the bucket runs with fewer pairs per CTA instead of failing."""
    rng = random.Random(60 + k + threads)
    us, vs = _skewed(rng, 0, 0, 30)
    for nb in (175000, 150000, 60000, 20000, 9000):
        a, b = _pair(rng, nb, rng.randint(1, nb // 3))
        us.append(a)
        vs.append(b)
    with mgcd.Device(0, 32) as dev:
        for cls in (0, 1, 2):
            dev.set_size_class(cls, threads, k, 1.0)
        assert mgcd.moduli_needed(175000) > 15000
        assert dev.gcd_batch(us, vs) == [math.gcd(a, b) for a, b in zip(us, vs)]


@pytest.mark.parametrize("cls_cfg", [{2: (1024, 4, 0.8, 4), 1: (1024, 4, 0.9, 2)}, {0: (512, 2, 1.0, 2), 2: (512, 4, 1.0, 8)}])
def test_size_classes_on_clusters(mgcd, cls_cfg):
    """Pairs of classes 0-2 spread over clusters of CTAs (k pairs per cluster)."""
    rng = random.Random(70 + len(cls_cfg))
    us, vs, _ = importlib.import_module("modgcd-onegpu_gb300.workloads").mixed_batch(300, seed=71)
    exp = [math.gcd(a, b) for a, b in zip(us, vs)]
    with mgcd.Device(0, 32) as dev:
        for c, (t, k, s, cs) in cls_cfg.items():
            dev.set_size_class(c, t, k, s)
            dev.set_class_cluster(c, cs)
            assert dev.get_class_cluster(c) == cs
        assert dev.gcd_batch(us, vs) == exp
        dev.batch_use_graph(True)
        dev.batch_upload(*mgcd.pack_pairs(us, vs))
        for _ in range(2):
            dev.batch_run()
            dev.batch_sync()
            assert _results(mgcd, dev) == exp


@pytest.mark.parametrize("L,scale", [(27, 0.76), (32, 0.8)])
def test_eight_pairs_per_cta(mgcd, L, scale):
    """K = 8 pairs per 1024-thread CTA share one inverse per modulus: the mixed batch (with
    scaled moduli counts, so some pairs may be rerun) gives every gcd exactly."""
    us, vs, _ = importlib.import_module("modgcd-onegpu_gb300.workloads").mixed_batch(400, seed=81)
    exp = [math.gcd(a, b) for a, b in zip(us, vs)]
    with mgcd.Device(0, L) as dev:
        for cls in (0, 1, 2):
            dev.set_size_class(cls, 1024, 8, scale)
        assert dev.gcd_batch(us, vs) == exp


def test_cta_trace_accounts_every_pair(mgcd):
    """The occupancy trace: one record per CTA of the run, every pair counted once, phases
    recorded for the K-slot CTAs, and the results unchanged with the trace on."""
    us, vs, _ = importlib.import_module("modgcd-onegpu_gb300.workloads").mixed_batch(300, seed=82)
    exp = [math.gcd(a, b) for a, b in zip(us, vs)]
    with mgcd.Device(0, 27) as dev:
        dev.load_tuning(mgcd.default_tuning_path(dev))
        dev.set_cta_trace(True)
        assert dev.gcd_batch(us, vs) == exp
        rec = dev.batch_cta_trace()
    assert len(rec) > 0 and (rec["ran"] != 0).all()
    assert int(rec["pairs"].sum()) == len(us)
    assert (rec["t_end_ms"] >= rec["t_start_ms"]).all()
    kslot = rec[rec["iterations"] > 0]
    assert len(kslot) > 0 and (kslot["cycles_update"] > 0).all()
