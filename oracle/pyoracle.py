"""Python binding of the oracle (test infrastructure only).

Loads ``liboracle.so`` (the C restatement of the reference algorithm) and
``libcpugmp.so`` (GMP ``mpz_gcd`` over a batch on the host cores).  Only the tests,
``__graft_entry__.smoke()`` and the CPU-baseline leg of ``bench.py`` import this module;
the product never does.

Integer conventions follow the reference's host code (GmpCudaDevice-gcd.cu:57-132):
operands are exported as little-endian 32-bit limbs, the larger one first.
"""
import ctypes
import os
import subprocess

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))

ORC_OK, ORC_ERR_REDUX, ORC_ERR_RECOVERY, ORC_ERR_ARG, ORC_ERR_CAPACITY, ORC_ERR_NOMEM = range(6)
MOD_INFINITY = -(1 << 31)


class Pair(ctypes.Structure):
    _fields_ = [("modulus", ctypes.c_uint32), ("value", ctypes.c_int32)]


_lib = None
_gmp = None


def build():
    """Compile the oracle libraries (``make -C oracle``)."""
    subprocess.run(["make", "-s", "-C", HERE, "all"], check=True)


def _load():
    global _lib
    if _lib is None:
        path = os.path.join(HERE, "liboracle.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        lib.orc_gen_moduli.restype = ctypes.c_size_t
        lib.orc_gen_moduli.argtypes = [ctypes.c_int, ctypes.c_void_p, ctypes.c_size_t]
        lib.orc_num_moduli_needed.restype = ctypes.c_int
        lib.orc_num_moduli_needed.argtypes = [ctypes.c_size_t, ctypes.c_int]
        lib.orc_residues.restype = None
        lib.orc_residues.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p]
        lib.orc_modgcd.restype = ctypes.c_int
        lib.orc_modgcd.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                   ctypes.c_void_p, ctypes.c_size_t,
                                   ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                   ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                   ctypes.POINTER(ctypes.c_size_t)]
        lib.orc_modgcd_grow.restype = ctypes.c_int
        lib.orc_modgcd_grow.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t, ctypes.c_int,
                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.c_size_t, ctypes.c_uint,
                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                        ctypes.c_void_p, ctypes.c_size_t, ctypes.POINTER(ctypes.c_size_t),
                                        ctypes.POINTER(ctypes.c_size_t), ctypes.POINTER(ctypes.c_size_t)]
        lib.orc_mixed_radix_to_limbs.restype = ctypes.c_long
        lib.orc_mixed_radix_to_limbs.argtypes = [ctypes.c_void_p, ctypes.c_size_t, ctypes.c_void_p, ctypes.c_size_t]
        _lib = lib
    return _lib


def _load_gmp():
    global _gmp
    if _gmp is None:
        path = os.path.join(HERE, "libcpugmp.so")
        if not os.path.exists(path):
            build()
        lib = ctypes.CDLL(path)
        lib.cpu_gmp_gcd_batch.restype = ctypes.c_int
        lib.cpu_gmp_gcd_batch.argtypes = [ctypes.c_size_t, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                          ctypes.c_int, ctypes.POINTER(ctypes.c_double)]
        lib.cpu_gmp_version.restype = ctypes.c_char_p
        _gmp = lib
    return _gmp


# ----------------------------------------------------------------- integer helpers ----

def to_limbs(x: int) -> np.ndarray:
    """Little-endian 32-bit limbs of x >= 0 (mpz_export(..., -1, 4, 0, 0, x)); 0 -> no limbs."""
    if x == 0:
        return np.zeros(0, dtype=np.uint32)
    n = (x.bit_length() + 31) // 32
    return np.frombuffer(x.to_bytes(4 * n, "little"), dtype="<u4").astype(np.uint32)


def from_limbs(a) -> int:
    a = np.ascontiguousarray(a, dtype="<u4")
    return int.from_bytes(a.tobytes(), "little")


# ------------------------------------------------------------------- the oracle ------

def gen_moduli(L: int, n: int) -> np.ndarray:
    """The first n moduli of the L-bit table (createModuli.cpp order)."""
    out = np.zeros(n, dtype=np.uint32)
    got = _load().orc_gen_moduli(L, out.ctypes.data, n)
    return out[:got]


def num_moduli_needed(bits: int, L: int) -> int:
    return _load().orc_num_moduli_needed(bits, L)


def residues(x: int, moduli: np.ndarray) -> np.ndarray:
    xl = to_limbs(x)
    out = np.zeros(len(moduli), dtype=np.uint32)
    m = np.ascontiguousarray(moduli, dtype=np.uint32)
    _load().orc_residues(xl.ctypes.data, len(xl), m.ctypes.data, len(m), out.ctypes.data)
    return out


def modgcd(u: int, v: int, L: int, moduli: np.ndarray, nq: int):
    """Runs the restated kernel on u >= v > 0 with the first nq moduli.

    Returns (status, digits, trace, iters): digits as a list of (modulus, value), trace the
    (p, b) pairs collected by the reduction loop (terminating pair included)."""
    ul, vl = to_limbs(u), to_limbs(v)
    m = np.ascontiguousarray(moduli[:nq], dtype=np.uint32)
    cap = nq + 2
    dig = (Pair * cap)()
    tr = (Pair * (nq + 2))()
    nd, nt, it = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
    st = _load().orc_modgcd(ul.ctypes.data, len(ul), vl.ctypes.data, len(vl), L, m.ctypes.data, nq,
                            dig, cap, ctypes.byref(nd), tr, nq + 2, ctypes.byref(nt), ctypes.byref(it))
    digits = [(dig[i].modulus, dig[i].value) for i in range(min(nd.value, cap))]
    trace = [(tr[i].modulus, tr[i].value) for i in range(min(nt.value, nq + 2))]
    return st, digits, trace, it.value


ORC_ERR_UNCERTIFIED = 6


def grow_start_count(ref: int, start: float) -> int:
    """A batched pair's first moduli count under growth (the plan's rounding: a multiple of
    32, at least 64, at most the reference count)."""
    n0 = (int(np.ceil(np.float32(start) * np.float32(ref))) + 31) // 32 * 32
    return min(ref, max(64, n0))


def grow_cap(ref: int) -> int:
    """The moduli a batched pair may grow to: the reference count plus a sixteenth, rounded
    up to 32, at most 16,384 (the K-slot kernels' limit)."""
    return max(ref, min(16384, (ref + ref // 16 + 31) // 32 * 32))


def modgcd_grow(u: int, v: int, L: int, moduli: np.ndarray, nq0: int, nq_cap: int, step_permille: int):
    """The restated loop with moduli grown on demand (orc_modgcd_grow) on u >= v > 0.

    Returns (status, digits, iters, nq_final)."""
    ul, vl = to_limbs(u), to_limbs(v)
    m = np.ascontiguousarray(moduli[:nq_cap], dtype=np.uint32)
    cap = nq_cap + 2
    dig = (Pair * cap)()
    nd, nt, it, nf = ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t(), ctypes.c_size_t()
    st = _load().orc_modgcd_grow(ul.ctypes.data, len(ul), vl.ctypes.data, len(vl), L, m.ctypes.data, nq0, nq_cap,
                                 step_permille, dig, cap, ctypes.byref(nd), None, 0, ctypes.byref(nt),
                                 ctypes.byref(it), ctypes.byref(nf))
    digits = [(dig[i].modulus, dig[i].value) for i in range(min(nd.value, cap))]
    return st, digits, it.value, nf.value


def mixed_radix_to_int(digits) -> int:
    """|g| from signed mixed-radix digits (GmpCudaDevice-gcd.cu:116-129), in Python."""
    if not digits:
        return 0
    g = digits[-1][1]
    for mod, val in reversed(digits[:-1]):
        g = g * mod + val
    return abs(g)


def mixed_radix_to_int_c(digits) -> int:
    """The same conversion through the C restatement."""
    n = len(digits)
    arr = (Pair * max(n, 1))()
    for i, (m, v) in enumerate(digits):
        arr[i].modulus, arr[i].value = m, v
    cap = n + 2
    out = np.zeros(cap, dtype=np.uint32)
    ln = _load().orc_mixed_radix_to_limbs(arr, n, out.ctypes.data, cap)
    assert ln >= 0
    return from_limbs(out[:ln])


class RefError(RuntimeError):
    """Mirrors the std::runtime_error strings of GmpCudaDevice-gcd.cu:76-111."""


def ref_gcd(u: int, v: int, L: int = 32, moduli=None, num_moduli: int = 65536, max_grid: int = 256):
    """The reference host entry GmpCudaDevice::gcd (GmpCudaDevice-gcd.cu:57-132) restated
    over the oracle: swap so u >= v, size the moduli, run, convert.  Raises RefError with
    the reference's messages.  Zero operands are outside the reference's domain and are
    rejected here."""
    if u < v:
        u, v = v, u
    if v <= 0:
        raise ValueError("oracle ref_gcd needs u >= v > 0")
    nq = num_moduli_needed(u.bit_length(), L)
    if nq > num_moduli:
        raise RefError("Not enough moduli available for given input.")
    if nq // 256 > max_grid:
        raise RefError("Cannot allocate enough threads to support computation.")
    if moduli is None:
        moduli = gen_moduli(L, nq)
    st, digits, _, _ = modgcd(u, v, L, moduli, nq)
    if st == ORC_ERR_REDUX:
        raise RefError("Ran out of moduli in the reduction loop.")
    if st == ORC_ERR_RECOVERY:
        raise RefError("Ran out of moduli in the recovery loop.")
    if st != ORC_OK:
        raise RefError("Unknown error in the gcd kernel.")
    return mixed_radix_to_int(digits)


# ------------------------------------------------------------ GMP batch (CPU) --------

def gmp_version() -> str:
    return _load_gmp().cpu_gmp_version().decode()


def cpu_gmp_gcd_batch(limbs, u_off, u_len, v_off, v_len, nthreads: int, want_results=True):
    """mpz_gcd of every pair of a packed batch on nthreads host threads.

    Returns (seconds, g_limbs, g_off, g_len); seconds covers the mpz_gcd calls only."""
    n = len(u_off)
    limbs = np.ascontiguousarray(limbs, dtype=np.uint32)
    u_off = np.ascontiguousarray(u_off, dtype=np.uint64)
    v_off = np.ascontiguousarray(v_off, dtype=np.uint64)
    u_len = np.ascontiguousarray(u_len, dtype=np.uint32)
    v_len = np.ascontiguousarray(v_len, dtype=np.uint32)
    g_cap = np.maximum(np.maximum(u_len, v_len), 1).astype(np.uint32)
    g_off = np.zeros(n, dtype=np.uint64)
    if n:
        g_off[1:] = np.cumsum(g_cap[:-1], dtype=np.uint64)
    g = np.zeros(int(g_cap.sum()) + 1, dtype=np.uint32)
    g_len = np.zeros(n, dtype=np.uint32)
    secs = ctypes.c_double()
    rc = _load_gmp().cpu_gmp_gcd_batch(n, limbs.ctypes.data, u_off.ctypes.data, u_len.ctypes.data,
                                       v_off.ctypes.data, v_len.ctypes.data,
                                       g.ctypes.data if want_results else None, g_off.ctypes.data,
                                       g_cap.ctypes.data, g_len.ctypes.data, int(nthreads), ctypes.byref(secs))
    if rc != 0:
        raise RuntimeError("cpu_gmp_gcd_batch: output capacity")
    return secs.value, g, g_off, g_len
