"""The request server (continuous batching under an HBM admission budget).

- Each result is the same alone (one request on an idle server) and in the mix (the same
  request among a Poisson stream of others of mixed sizes), and equals Python's gcd.
- Continuous lanes take requests into running kernels (far fewer launches than requests)
  and answer exactly what the wave path answers.
- The admission budget is never exceeded and an oversize request is refused.
- While a server runs, the context's own calls are refused; afterwards they work again.
"""
import importlib
import math
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu

wl = importlib.import_module("modgcd-onegpu_gb300.workloads")


def _cap(u, v):
    return max(u.bit_length(), v.bit_length()) // 32 + 2


def test_same_alone_and_in_the_mix(mgcd):
    us, vs, arr = wl.serve_requests(400, 20000.0, seed=7, big_frac=0.01, big_bits=150000, hi_bits=16384)
    us += [0, 12345, 7 * 2**5000]          # zero operands and a tiny pair ride along
    vs += [99, 0, 7 * 3**3000]
    arr += [arr[-1] + 1e-4] * 3
    exp = [math.gcd(u, v) for u, v in zip(us, vs)]
    with mgcd.Device(0, 32) as dev:
        with mgcd.Server(dev) as srv:
            alone = [srv.gcd(u, v) for u, v in zip(us, vs)]
            mix, st, lat, makespan = srv.replay(us, vs, arr)
            stats = srv.stats()
        assert alone == exp
        assert mix == exp
        assert (st == 0).all()
        assert (lat > 0).all() and makespan >= max(arr)
        assert stats["completed"] == 2 * len(us)
        # in the mix, requests share waves: far fewer waves than requests
        assert stats["waves"] < 2 * len(us)


def test_admission_budget(mgcd):
    rng = random.Random(8)
    budget = 600_000
    with mgcd.Device(0, 32) as dev:
        with mgcd.Server(dev, budget_bytes=budget) as srv:
            big = rng.getrandbits(400000) | 1
            with pytest.raises(mgcd.GcdError) as e:
                srv.submit(big, big + 2)
            assert mgcd.STATUS_NAMES[e.value.status] == "MGCD_ERR_BUDGET"
            us = [rng.getrandbits(rng.randint(1000, 20000)) | 1 for _ in range(300)]
            vs = [rng.getrandbits(rng.randint(1000, 20000)) | 1 for _ in range(300)]
            tickets = [srv.submit(u, v) for u, v in zip(us, vs)]
            got = [srv.take(t, _cap(u, v))[0] for t, u, v in zip(tickets, us, vs)]
            stats = srv.stats()
        assert got == [math.gcd(u, v) for u, v in zip(us, vs)]
        assert 0 < stats["peak_admitted_bytes"] <= budget
        assert stats["launches"] > 1


def test_take_timeout_keeps_the_ticket(mgcd):
    rng = random.Random(9)
    g = rng.getrandbits(60000) | 1
    u, v = g * (rng.getrandbits(200000) | 1), g * (rng.getrandbits(200000) | 1)
    with mgcd.Device(0, 32) as dev:
        with mgcd.Server(dev) as srv:
            t = srv.submit(u, v)
            with pytest.raises(mgcd.GcdError) as e:
                srv.take(t, _cap(u, v), timeout_ms=1)
            assert mgcd.STATUS_NAMES[e.value.status] == "MGCD_ERR_TIMEOUT"
            assert srv.take(t, _cap(u, v))[0] == math.gcd(u, v)
            with pytest.raises(mgcd.GcdError):      # released
                srv.poll(t)


def test_context_refuses_direct_calls_while_serving(mgcd):
    with mgcd.Device(0, 32) as dev:
        srv = mgcd.Server(dev)
        with pytest.raises(mgcd.GcdError) as e:
            dev.gcd(6, 4)
        assert mgcd.STATUS_NAMES[e.value.status] == "MGCD_ERR_BUSY"
        with pytest.raises(mgcd.GcdError):
            mgcd.Server(dev)
        srv.close()
        assert dev.gcd(6, 4) == 2


def test_many_threads_submit_and_take(mgcd):
    """Submissions and takes from several host threads at once: every answer is exact and
    belongs to its own request."""
    import threading
    results, errors = {}, []
    with mgcd.Device(0, 32) as dev:
        with mgcd.Server(dev) as srv:
            def worker(tid):
                try:
                    rng = random.Random(1000 + tid)
                    mine = []
                    for _ in range(60):
                        nb = rng.randint(500, 20000)
                        g = rng.getrandbits(rng.randint(1, nb // 2)) | 1
                        u, v = g * (rng.getrandbits(nb) | 1), g * (rng.getrandbits(nb) | 1)
                        mine.append((srv.submit(u, v), u, v))
                    for t, u, v in mine:
                        results[t] = (srv.take(t, _cap(u, v))[0], math.gcd(u, v))
                except Exception as e:   # surfaced by the assertion below
                    errors.append(e)
            ths = [threading.Thread(target=worker, args=(i,)) for i in range(6)]
            for th in ths:
                th.start()
            for th in ths:
                th.join()
    assert not errors, errors
    assert len(results) == 360
    assert all(got == exp for got, exp in results.values())


def test_continuous_lanes_take_requests_while_running(mgcd):
    """Requests arriving over ~40 ms (Poisson at 10k req/s, 1k-16k bits) are taken by the
    lanes' running kernels as their slots free up: far fewer kernel launches than requests,
    no wave at all, and every answer equals the wave path's and Python's gcd."""
    us, vs, arr = wl.serve_requests(400, 10000.0, seed=17, big_frac=0.0, hi_bits=16384)
    exp = [math.gcd(u, v) for u, v in zip(us, vs)]
    with mgcd.Device(0, 32) as dev:
        with mgcd.Server(dev) as srv:
            got, st, lat, _ = srv.replay(us, vs, arr)
            stats = srv.stats()
        with mgcd.Server(dev) as srv:
            srv.set_continuous(False)
            got_w, st_w, _, _ = srv.replay(us, vs, arr)
            stats_w = srv.stats()
    assert got == exp and got_w == exp
    assert (st == 0).all() and (st_w == 0).all()
    assert stats["waves"] == 0 and 0 < stats["launches"] < len(us) // 4
    assert stats_w["waves"] > 0


def test_continuous_lanes_rerun_uncertified_pairs(mgcd):
    """With moduli counts scaled far below the reference's, many requests cannot be
    certified; the continuous lanes rerun them with the reference count and every answer
    stays exact."""
    us, vs, arr = wl.serve_requests(200, 20000.0, seed=18, big_frac=0.0, hi_bits=30000)
    with mgcd.Device(0, 32) as dev:
        dev.set_nq_scale(0.5)
        with mgcd.Server(dev) as srv:
            got, st, _, _ = srv.replay(us, vs, arr)
    assert (st == 0).all()
    assert got == [math.gcd(u, v) for u, v in zip(us, vs)]
