"""Seeded synthetic gcd workloads with the shapes of the benchmark workloads.

No public dataset is involved: the reference generates its inputs with GMP's Mersenne
Twister (testmodgcd.cpp:219-229, u = g*a, v = g*b from mpz_urandomb); these generators draw
uniform random limbs the same way from Python's seeded Mersenne Twister.

  single_pair      one pair: g 2048-bit odd, a, b 8192-bit coprime, u = g*a, v = g*b
  size_sweep_pair  n-bit operands with an n/4-bit planted gcd
  mixed_batch      4096 pairs, bits(u) log-uniform in [1k, 64k], bits(v) = bits(u)/U(1, 2);
                   25% coprime, 5% v | u, 70% planted gcd of U[0, 50%] of the smaller operand
  skewed_batch     64 pairs at 1M bits + 16384 pairs of U[512, 4096] bits
  serve_requests   Poisson arrivals, mixed-batch sizes plus 1% 1M-bit requests
"""
import math
import random


def _rand_bits(rng, n):
    """Uniform n-bit integer with the top bit set (n >= 1)."""
    return rng.getrandbits(n) | (1 << (n - 1))


def single_pair(seed=1):
    rng = random.Random(seed)
    g = _rand_bits(rng, 2048) | 1
    while True:
        a, b = _rand_bits(rng, 8192), _rand_bits(rng, 8192)
        if math.gcd(a, b) == 1:
            return g * a, g * b


def size_sweep_pair(nbits, seed=1, gcd_frac=0.25):
    rng = random.Random(seed * 1000003 + nbits)
    gb = max(1, int(nbits * gcd_frac))
    g = _rand_bits(rng, gb)
    return g * _rand_bits(rng, nbits - gb), g * _rand_bits(rng, nbits - gb)


def mixed_pair(rng, lo_bits=1024, hi_bits=65536):
    bu = int(round(2 ** rng.uniform(math.log2(lo_bits), math.log2(hi_bits))))
    bv = max(2, int(round(bu / rng.uniform(1.0, 2.0))))
    r = rng.random()
    if r < 0.25:                                   # coprime
        a = _rand_bits(rng, bu)
        while True:
            b = _rand_bits(rng, bv)
            if math.gcd(a, b) == 1:
                return a, b, "coprime"
    if r < 0.30:                                   # v divides u
        v = _rand_bits(rng, bv)
        c = _rand_bits(rng, max(1, bu - bv))
        return v * c, v, "divides"
    gb = int(rng.uniform(0.0, 0.5) * min(bu, bv))  # planted gcd
    g = _rand_bits(rng, gb) if gb > 0 else 1
    return g * _rand_bits(rng, bu - gb), g * _rand_bits(rng, bv - gb), "planted"


def mixed_batch(n=4096, seed=3, lo_bits=1024, hi_bits=65536):
    rng = random.Random(seed)
    us, vs, kinds = [], [], []
    for _ in range(n):
        u, v, k = mixed_pair(rng, lo_bits, hi_bits)
        us.append(u)
        vs.append(v)
        kinds.append(k)
    return us, vs, kinds


def serve_requests(n, rate, seed=5, big_frac=0.01, big_bits=1 << 20, lo_bits=1024, hi_bits=65536):
    """Open-loop serving load: n requests with Poisson arrivals at `rate` per second
    (exponential gaps, seeded), sizes from the mixed-batch distribution plus a `big_frac`
    share of big_bits-bit requests (planted gcd of U[0, 50%]).  Returns (us, vs, arrival_s).
    The big requests sit at evenly spread positions so every prefix has its share."""
    rng = random.Random(seed)
    us, vs, arr = [], [], []
    t = 0.0
    n_big = int(round(n * big_frac))
    big_at = {int((k + 0.5) * n / n_big) for k in range(n_big)} if n_big else set()
    for i in range(n):
        t += rng.expovariate(rate)
        arr.append(t)
        if i in big_at:
            gb = int(rng.uniform(0.0, 0.5) * big_bits)
            g = _rand_bits(rng, gb) if gb > 0 else 1
            us.append(g * _rand_bits(rng, big_bits - gb))
            vs.append(g * _rand_bits(rng, big_bits - gb))
        else:
            u, v, _ = mixed_pair(rng, lo_bits, hi_bits)
            us.append(u)
            vs.append(v)
    return us, vs, arr


def skewed_batch(n_big=64, big_bits=1 << 20, n_small=16384, seed=4):
    rng = random.Random(seed)
    us, vs = [], []
    for _ in range(n_big):
        gb = rng.randint(1, big_bits // 2)
        g = _rand_bits(rng, gb)
        us.append(g * _rand_bits(rng, big_bits - gb))
        vs.append(g * _rand_bits(rng, big_bits - gb))
    for _ in range(n_small):
        nb = rng.randint(512, 4096)
        gb = rng.randint(1, nb // 2)
        g = _rand_bits(rng, gb)
        us.append(g * _rand_bits(rng, nb - gb))
        vs.append(g * _rand_bits(rng, max(2, rng.randint(nb // 2, nb) - gb)))
    return us, vs
