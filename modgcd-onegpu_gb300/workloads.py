"""Seeded synthetic gcd workloads with the shapes of the benchmark workloads.

No public dataset is involved: the reference generates its inputs with GMP's Mersenne
Twister (testmodgcd.cpp:159-160, 219-229: gmp_randinit_mt, then u, v and g from
mpz_urandomb, u *= g, v *= g), and so do these generators, through the system's GMP
runtime (libgmp.so.10): every operand limb is an mpz_urandomb draw, and the sizes, mixes
and arrival gaps come from the same stream (53-bit mpz_urandomb draws as uniform floats).
`reference_pairs` reproduces the reference driver's own stream exactly (its test-vector
files); the configurations below draw in the same order with their own constraints (top
bits set to fix the bit lengths, odd or coprime factors where the configuration says so).

  single_pair      one pair: g 2048-bit odd, a, b 8192-bit coprime, u = g*a, v = g*b
  size_sweep_pair  n-bit operands with an n/4-bit planted gcd
  mixed_batch      4096 pairs, bits(u) log-uniform in [1k, 64k], bits(v) = bits(u)/U(1, 2);
                   25% coprime, 5% v | u, 70% planted gcd of U[0, 50%] of the smaller operand
  skewed_batch     64 pairs at 1M bits + 16384 pairs of U[512, 4096] bits
  serve_requests   Poisson arrivals, mixed-batch sizes plus 1% 1M-bit requests
"""
import ctypes
import math


class _Mpz(ctypes.Structure):
    # mpz_t as the GMP manual documents it ("Integer Internals")
    _fields_ = [("alloc", ctypes.c_int), ("size", ctypes.c_int), ("d", ctypes.c_void_p)]


class _Gmp:
    """The libgmp.so.10 entry points used here (exported as __gmpz_* / __gmp_*)."""

    def __init__(self):
        lib = ctypes.CDLL("libgmp.so.10")

        def fn(name, argtypes, restype=None):
            f = getattr(lib, name)
            f.argtypes = argtypes
            f.restype = restype
            return f
        P = ctypes.POINTER(_Mpz)
        self.mpz_init = fn("__gmpz_init", [P])
        self.mpz_clear = fn("__gmpz_clear", [P])
        self.mpz_urandomb = fn("__gmpz_urandomb", [P, ctypes.c_void_p, ctypes.c_ulong])
        self.mpz_export = fn("__gmpz_export", [ctypes.c_void_p, ctypes.POINTER(ctypes.c_size_t), ctypes.c_int,
                                               ctypes.c_size_t, ctypes.c_int, ctypes.c_size_t, P], ctypes.c_void_p)
        self.randinit_mt = fn("__gmp_randinit_mt", [ctypes.c_void_p])
        self.randseed_ui = fn("__gmp_randseed_ui", [ctypes.c_void_p, ctypes.c_ulong])
        self.randclear = fn("__gmp_randclear", [ctypes.c_void_p])


_gmp = None


def _libgmp():
    global _gmp
    if _gmp is None:
        _gmp = _Gmp()
    return _gmp


class GmpRandom:
    """GMP's Mersenne Twister: gmp_randinit_mt, then gmp_randseed_ui(seed) unless seed is
    None (GMP's default seed, as the reference's driver uses it)."""

    def __init__(self, seed=None):
        self._g = _libgmp()
        self._state = ctypes.create_string_buffer(256)      # gmp_randstate_t (opaque, < 64 bytes)
        self._g.randinit_mt(self._state)
        if seed is not None:
            self._g.randseed_ui(self._state, seed)
        self._z = _Mpz()
        self._g.mpz_init(ctypes.byref(self._z))

    def __del__(self):
        try:
            self._g.mpz_clear(ctypes.byref(self._z))
            self._g.randclear(self._state)
        except (AttributeError, TypeError):
            pass

    def urandomb(self, n):
        """mpz_urandomb(state, n): uniform in [0, 2^n)."""
        if n <= 0:
            return 0
        self._g.mpz_urandomb(ctypes.byref(self._z), self._state, n)
        buf = ctypes.create_string_buffer((n + 7) // 8 + 8)
        cnt = ctypes.c_size_t(0)
        self._g.mpz_export(buf, ctypes.byref(cnt), -1, 1, 0, 0, ctypes.byref(self._z))
        return int.from_bytes(buf.raw[: cnt.value], "little")

    def random(self):
        """Uniform float in [0, 1) from a 53-bit draw."""
        return self.urandomb(53) / float(1 << 53)

    def uniform(self, a, b):
        return a + (b - a) * self.random()

    def randint(self, a, b):
        """Uniform integer in [a, b]."""
        return a + min(b - a, int(self.random() * (b - a + 1)))

    def expovariate(self, rate):
        return -math.log(1.0 - self.random()) / rate


def reference_pairs(num_bits, num_g_bits, count, seed=None):
    """The pairs the reference's test driver draws (testmodgcd.cpp:219-229): u, v of
    num_bits - num_g_bits random bits and g of num_g_bits (each redrawn while zero), then
    u *= g, v *= g -- the contents of its tests/<bits>-<gbits> files for a fresh stream."""
    rng = GmpRandom(seed)

    def nonzero(n):
        while True:
            x = rng.urandomb(n)
            if x:
                return x
    out = []
    for _ in range(count):
        u = nonzero(num_bits - num_g_bits)
        v = nonzero(num_bits - num_g_bits)
        g = nonzero(num_g_bits)
        out.append((g * u, g * v))
    return out


def _rand_bits(rng, n):
    """Uniform n-bit integer with the top bit set (n >= 1)."""
    return rng.urandomb(n) | (1 << (n - 1))


def single_pair(seed=1):
    """Drawn in the reference driver's order (a, b, then g); a new (a, b) while not coprime."""
    rng = GmpRandom(seed)
    while True:
        a, b = _rand_bits(rng, 8192), _rand_bits(rng, 8192)
        g = _rand_bits(rng, 2048) | 1
        if math.gcd(a, b) == 1:
            return g * a, g * b


def size_sweep_pair(nbits, seed=1, gcd_frac=0.25):
    rng = GmpRandom(seed * 1000003 + nbits)
    gb = max(1, int(nbits * gcd_frac))
    a, b = _rand_bits(rng, nbits - gb), _rand_bits(rng, nbits - gb)
    g = _rand_bits(rng, gb)
    return g * a, g * b


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
    a, b = _rand_bits(rng, bu - gb), _rand_bits(rng, bv - gb)
    g = _rand_bits(rng, gb) if gb > 0 else 1
    return g * a, g * b, "planted"


def mixed_batch(n=4096, seed=3, lo_bits=1024, hi_bits=65536):
    rng = GmpRandom(seed)
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
    rng = GmpRandom(seed)
    us, vs, arr = [], [], []
    t = 0.0
    n_big = int(round(n * big_frac))
    big_at = {int((k + 0.5) * n / n_big) for k in range(n_big)} if n_big else set()
    for i in range(n):
        t += rng.expovariate(rate)
        arr.append(t)
        if i in big_at:
            gb = int(rng.uniform(0.0, 0.5) * big_bits)
            a, b = _rand_bits(rng, big_bits - gb), _rand_bits(rng, big_bits - gb)
            g = _rand_bits(rng, gb) if gb > 0 else 1
            us.append(g * a)
            vs.append(g * b)
        else:
            u, v, _ = mixed_pair(rng, lo_bits, hi_bits)
            us.append(u)
            vs.append(v)
    return us, vs, arr


def skewed_batch(n_big=64, big_bits=1 << 20, n_small=16384, seed=4):
    rng = GmpRandom(seed)
    us, vs = [], []
    for _ in range(n_big):
        gb = rng.randint(1, big_bits // 2)
        a, b = _rand_bits(rng, big_bits - gb), _rand_bits(rng, big_bits - gb)
        g = _rand_bits(rng, gb)
        us.append(g * a)
        vs.append(g * b)
    for _ in range(n_small):
        nb = rng.randint(512, 4096)
        gb = rng.randint(1, nb // 2)
        a = _rand_bits(rng, nb - gb)
        b = _rand_bits(rng, max(2, rng.randint(nb // 2, nb) - gb))
        g = _rand_bits(rng, gb)
        us.append(g * a)
        vs.append(g * b)
    return us, vs
