"""GB300 modular integer GCD -- Python binding of the C ABI (include/modgcd.h, libmodgcd.so).

Mirrors the reference's host object GmpCuda::GmpCudaDevice (GmpCuda.h:87-119):

    Device.set_device(0)          GmpCudaDevice::setDevice     (GmpCudaDevice.cu:96-103)
    dev = Device()                GmpCudaDevice()              (GmpCudaDevice.cu:107-137)
    dev.gcd(u, v)                 GmpCudaDevice::gcd           (GmpCudaDevice-gcd.cu:57-132)
    dev.max_grid_size             getMaxGridSize               (GmpCuda.h:118)

plus batches (``gcd_batch`` and the upload/run/download steps, CUDA-graph replay, the
tuning table), the request server (``Server``: continuous batching under an HBM admission
budget) and the exhaustive inverse certification.  Errors raise ``GcdError`` with the
reference's messages.  Every computation runs on the GPU through libmodgcd.so; there is
no CPU path, and loading fails loudly if the library is missing.
"""
import ctypes
import os

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
LIB_DIR = os.path.join(HERE, "lib")
LIB_PATH = os.path.join(LIB_DIR, "libmodgcd.so")

MGCD_OK = 0
MGCD_ERR_NO_DEVICE = 2
MGCD_ERR_CAPACITY = 10
STATUS_NAMES = {
    0: "MGCD_OK", 1: "MGCD_ERR_INVALID_ARG", 2: "MGCD_ERR_NO_DEVICE", 3: "MGCD_ERR_CUDA",
    4: "MGCD_ERR_NOT_ENOUGH_MODULI", 5: "MGCD_ERR_GRID", 6: "MGCD_ERR_REDUX", 7: "MGCD_ERR_RECOVERY",
    8: "MGCD_ERR_KERNEL", 9: "MGCD_ERR_TIMEOUT", 10: "MGCD_ERR_CAPACITY", 11: "MGCD_ERR_BUDGET",
    12: "MGCD_ERR_BUSY",
}

# Every function declared in include/modgcd.h, with its ctypes signature.
_c = ctypes
_P = _c.c_void_p
SIGNATURES = {
    "mgcd_status_string": (_c.c_char_p, [_c.c_int]),
    "mgcd_device_count": (_c.c_int, [_c.POINTER(_c.c_int)]),
    "mgcd_set_device": (_c.c_int, [_c.c_int]),
    "mgcd_create": (_c.c_int, [_c.c_int, _c.c_int, _c.POINTER(_P)]),
    "mgcd_destroy": (_c.c_int, [_P]),
    "mgcd_max_grid_size": (_c.c_int, [_P, _c.POINTER(_c.c_int)]),
    "mgcd_num_moduli": (_c.c_int, [_P, _c.POINTER(_c.c_size_t)]),
    "mgcd_moduli": (_c.c_int, [_P, _P, _c.c_size_t]),
    "mgcd_moduli_needed": (_c.c_int, [_c.c_int, _c.c_size_t]),
    "mgcd_gen_moduli": (_c.c_size_t, [_c.c_int, _P, _c.c_size_t]),
    "mgcd_gcd_digits": (_c.c_int, [_P, _P, _c.c_size_t, _P, _c.c_size_t, _P, _c.c_size_t,
                                   _c.POINTER(_c.c_size_t)]),
    "mgcd_gcd": (_c.c_int, [_P, _P, _c.c_size_t, _P, _c.c_size_t, _P, _c.c_size_t, _c.POINTER(_c.c_size_t)]),
    "mgcd_gcd_batch": (_c.c_int, [_P, _c.c_size_t, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P]),
    "mgcd_batch_upload": (_c.c_int, [_P, _c.c_size_t, _P, _P, _P, _P, _P]),
    "mgcd_batch_run": (_c.c_int, [_P]),
    "mgcd_batch_sync": (_c.c_int, [_P]),
    "mgcd_batch_download": (_c.c_int, [_P, _P, _P, _P, _P, _P]),
    "mgcd_batch_launches": (_c.c_int, [_P, _c.POINTER(_c.c_int)]),
    "mgcd_batch_work": (_c.c_int, [_P, _c.POINTER(_c.c_double), _c.POINTER(_c.c_double),
                                   _c.POINTER(_c.c_double), _c.POINTER(_c.c_double)]),
    "mgcd_batch_alg_bytes": (_c.c_int, [_P, _c.POINTER(_c.c_double)]),
    "mgcd_set_cta_trace": (_c.c_int, [_P, _c.c_int]),
    "mgcd_batch_cta_trace": (_c.c_int, [_P, _P, _c.c_size_t, _c.POINTER(_c.c_size_t)]),
    "mgcd_batch_elapsed_ms": (_c.c_int, [_P, _c.POINTER(_c.c_float), _c.POINTER(_c.c_float),
                                         _c.POINTER(_c.c_int)]),
    "mgcd_batch_transfer_bytes": (_c.c_int, [_P, _c.POINTER(_c.c_uint64), _c.POINTER(_c.c_uint64)]),
    "mgcd_int_peak": (_c.c_int, [_P, _c.POINTER(_c.c_double)]),
    "mgcd_gcd_digits_noalloc": (_c.c_int, [_P, _c.c_size_t, _c.c_size_t, _P, _c.c_size_t, _P, _P, _P]),
    "mgcd_set_nq_scale": (_c.c_int, [_P, _c.c_float]),
    "mgcd_set_size_class": (_c.c_int, [_P, _c.c_int, _c.c_int, _c.c_int, _c.c_float]),
    "mgcd_set_single_pair_policy": (_c.c_int, [_P, _c.c_int]),
    "mgcd_set_wait_timeout_ms": (_c.c_int, [_P, _c.c_uint]),
    "mgcd_test_withhold_cta": (_c.c_int, [_P, _c.c_int]),
    "mgcd_test_fail_staging": (_c.c_int, [_P, _c.c_int]),
    "mgcd_test_force_moduli": (_c.c_int, [_P, _c.c_uint]),
    "mgcd_get_size_class": (_c.c_int, [_P, _c.c_int, _c.POINTER(_c.c_int), _c.POINTER(_c.c_int),
                                       _c.POINTER(_c.c_float)]),
    "mgcd_batch_kernel_stats": (_c.c_int, [_P, _c.c_int, _c.POINTER(_c.c_int), _c.POINTER(_c.c_int),
                                           _c.POINTER(_c.c_float)]),
    "mgcd_batch_retried": (_c.c_int, [_P, _c.POINTER(_c.c_int)]),
    "mgcd_batch_kernel_work": (_c.c_int, [_P, _c.c_int, _c.POINTER(_c.c_double), _c.POINTER(_c.c_double),
                                          _c.POINTER(_c.c_double), _c.POINTER(_c.c_double)]),
    "mgcd_set_cluster_size": (_c.c_int, [_P, _c.c_int]),
    "mgcd_get_cluster_size": (_c.c_int, [_P, _c.POINTER(_c.c_int)]),
    "mgcd_batch_use_graph": (_c.c_int, [_P, _c.c_int]),
    "mgcd_set_class_cluster": (_c.c_int, [_P, _c.c_int, _c.c_int]),
    "mgcd_get_class_cluster": (_c.c_int, [_P, _c.c_int, _c.POINTER(_c.c_int)]),
    "mgcd_certify_inverse": (_c.c_int, [_P, _c.POINTER(_c.c_uint64), _c.POINTER(_c.c_uint64),
                                        _c.POINTER(_c.c_uint32), _c.POINTER(_c.c_uint32)]),
    "mgcd_load_tuning": (_c.c_int, [_P, _c.c_char_p]),
    "mgcd_save_tuning": (_c.c_int, [_P, _c.c_char_p]),
    "mgcd_serve_start": (_c.c_int, [_P, _c.c_size_t, _P]),
    "mgcd_serve_set_continuous": (_c.c_int, [_P, _c.c_int]),
    "mgcd_serve_stop": (_c.c_int, [_P]),
    "mgcd_serve_submit": (_c.c_int, [_P, _P, _c.c_size_t, _P, _c.c_size_t, _c.POINTER(_c.c_uint64)]),
    "mgcd_serve_poll": (_c.c_int, [_P, _c.c_uint64, _c.POINTER(_c.c_int)]),
    "mgcd_serve_take": (_c.c_int, [_P, _c.c_uint64, _c.c_uint, _P, _c.c_size_t, _c.POINTER(_c.c_size_t),
                                   _c.POINTER(_c.c_double)]),
    "mgcd_serve_replay": (_c.c_int, [_P, _c.c_size_t, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P, _P,
                                     _c.POINTER(_c.c_double)]),
    "mgcd_serve_stats": (_c.c_int, [_P, _c.POINTER(_c.c_uint64), _c.POINTER(_c.c_uint64),
                                    _c.POINTER(_c.c_uint64), _c.POINTER(_c.c_uint64)]),
    "mgcd_serve_trace": (_c.c_int, [_P, _P, _c.c_size_t, _c.POINTER(_c.c_size_t)]),
    "mgcd_set_growth": (_c.c_int, [_P, _c.c_float, _c.c_uint]),
    "mgcd_get_growth": (_c.c_int, [_P, _c.POINTER(_c.c_float), _c.POINTER(_c.c_uint)]),
    "mgcd_batch_pair_digits": (_c.c_int, [_P, _c.c_size_t, _P, _c.c_size_t, _c.POINTER(_c.c_size_t),
                                          _c.POINTER(_c.c_uint32)]),
}

_lib = None


class GcdError(RuntimeError):
    """A failed call; ``status`` is the MGCD_* code, the message the reference's text."""

    def __init__(self, status, msg):
        super().__init__(msg)
        self.status = status


def load():
    """Loads libmodgcd.so (built in-tree by build.py) and declares its signatures."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise ImportError("libmodgcd.so is not built (%s): run modgcd-onegpu_gb300/build.py" % LIB_PATH)
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib


def status_string(code):
    return load().mgcd_status_string(int(code)).decode()


def _check(code):
    if code != MGCD_OK:
        raise GcdError(code, status_string(code))


def _ptr(a):
    return a.ctypes.data if a is not None and a.size else None


# ------------------------------------------------------------------ integers <-> limbs ----

def to_limbs(x):
    """|x| as little-endian uint32 limbs (mpz_export(..., -1, 4, 0, 0, x)); 0 -> empty."""
    x = abs(int(x))
    if x == 0:
        return np.zeros(0, dtype=np.uint32)
    n = (x.bit_length() + 31) // 32
    return np.frombuffer(x.to_bytes(4 * n, "little"), dtype="<u4").astype(np.uint32)


def from_limbs(a):
    return int.from_bytes(np.ascontiguousarray(a, dtype="<u4").tobytes(), "little")


def pack_pairs(us, vs):
    """Packs operand pairs into the batch layout: (limbs, u_off, u_len, v_off, v_len)."""
    parts, uo, ul, vo, vl = [], [], [], [], []
    off = 0
    for u, v in zip(us, vs):
        a, b = to_limbs(u), to_limbs(v)
        uo.append(off); ul.append(len(a)); parts.append(a); off += len(a)
        vo.append(off); vl.append(len(b)); parts.append(b); off += len(b)
    limbs = np.concatenate(parts) if parts else np.zeros(0, dtype=np.uint32)
    return (np.ascontiguousarray(limbs, dtype=np.uint32), np.array(uo, dtype=np.uint64),
            np.array(ul, dtype=np.uint32), np.array(vo, dtype=np.uint64), np.array(vl, dtype=np.uint32))


def result_layout(u_len, v_len):
    """Output capacity per pair (max operand size + 1) and offsets."""
    cap = (np.maximum(u_len, v_len).astype(np.uint64) + 1).astype(np.uint32)
    off = np.zeros(len(cap), dtype=np.uint64)
    if len(cap):
        off[1:] = np.cumsum(cap[:-1], dtype=np.uint64)
    return off, cap, int(cap.sum(dtype=np.uint64))


def moduli_needed(bits, L=32):
    return load().mgcd_moduli_needed(int(L), int(bits))


def gen_moduli(L, count):
    out = np.zeros(count, dtype=np.uint32)
    n = load().mgcd_gen_moduli(int(L), out.ctypes.data, count)
    return out[:n]


TUNING_DIR = os.path.join(HERE, "tuning")


def default_tuning_path(dev):
    """The committed tuning table for this modulus width on GB300 (written by tune.py)."""
    return os.path.join(TUNING_DIR, "gb300_L%d.txt" % dev.L)


def tuned_width(default=32):
    """Modulus width with the fastest whole mixed batch on GB300 (tune.py --compare-widths
    writes tuning/gb300_width.txt); `default` when no comparison was recorded."""
    try:
        with open(os.path.join(TUNING_DIR, "gb300_width.txt")) as f:
            L = int(f.readline().split()[0])
        return L if L in (22, 27, 32) else default
    except (OSError, ValueError, IndexError):
        return default


def device_count():
    n = ctypes.c_int()
    _check(load().mgcd_device_count(ctypes.byref(n)))
    return n.value


class Device:
    """One context (moduli table resident on the GPU) -- GmpCuda::GmpCudaDevice."""

    @staticmethod
    def set_device(dev_no=0):
        rc = load().mgcd_set_device(int(dev_no))
        if rc == MGCD_ERR_NO_DEVICE:
            raise GcdError(rc, "Invalid device number.")
        _check(rc)

    def __init__(self, device=-1, L=32):
        self._lib = load()
        self.L = L
        h = ctypes.c_void_p()
        _check(self._lib.mgcd_create(int(device), int(L), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mgcd_destroy(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    @property
    def max_grid_size(self):
        n = ctypes.c_int()
        _check(self._lib.mgcd_max_grid_size(self._h, ctypes.byref(n)))
        return n.value

    @property
    def num_moduli(self):
        n = ctypes.c_size_t()
        _check(self._lib.mgcd_num_moduli(self._h, ctypes.byref(n)))
        return n.value

    def moduli(self, n):
        out = np.zeros(n, dtype=np.uint32)
        _check(self._lib.mgcd_moduli(self._h, out.ctypes.data, n))
        return out

    def gcd(self, u, v):
        """gcd(u, v) of two Python integers (signs ignored)."""
        a, b = to_limbs(u), to_limbs(v)
        cap = max(len(a), len(b)) + 1
        g = np.zeros(cap, dtype=np.uint32)
        n = ctypes.c_size_t()
        _check(self._lib.mgcd_gcd(self._h, _ptr(a), len(a), _ptr(b), len(b), g.ctypes.data, cap, ctypes.byref(n)))
        return from_limbs(g[: n.value])

    def gcd_digits(self, u, v):
        """The signed mixed-radix digits [(modulus, value), ...] the kernel returns."""
        a, b = to_limbs(u), to_limbs(v)
        cap = moduli_needed(max(abs(u), abs(v)).bit_length(), self.L) + 2
        d = np.zeros(cap, dtype=[("modulus", "<u4"), ("value", "<i4")])
        n = ctypes.c_size_t()
        _check(self._lib.mgcd_gcd_digits(self._h, _ptr(a), len(a), _ptr(b), len(b), d.ctypes.data, cap,
                                         ctypes.byref(n)))
        return [(int(m), int(x)) for m, x in d[: n.value]]

    # ------------------------------------------------------------------ batches ----
    def gcd_batch(self, us, vs, return_status=False):
        """[gcd(u, v) for u, v in zip(us, vs)] in one batched run."""
        packed = pack_pairs(us, vs)
        g, g_off, g_len, st = self.gcd_batch_packed(*packed)
        res = [from_limbs(g[int(o): int(o) + int(n)]) for o, n in zip(g_off, g_len)]
        if return_status:
            return res, st
        bad = np.nonzero(st != MGCD_OK)[0]
        if len(bad):
            raise GcdError(int(st[bad[0]]), status_string(int(st[bad[0]])))
        return res

    def gcd_batch_packed(self, limbs, u_off, u_len, v_off, v_len, out=None):
        """mgcd_gcd_batch on packed pairs; `out` = (g, g_off, g_cap, g_len, status) arrays to
        reuse (sized by result_layout), else new ones."""
        n = len(u_off)
        if out is None:
            g_off, g_cap, tot = result_layout(u_len, v_len)
            g = np.zeros(max(tot, 1), dtype=np.uint32)
            g_len = np.zeros(n, dtype=np.uint32)
            st = np.zeros(n, dtype=np.int32)
        else:
            g, g_off, g_cap, g_len, st = out
        self._lib.mgcd_gcd_batch(self._h, n, _ptr(limbs), _ptr(u_off), _ptr(u_len), _ptr(v_off), _ptr(v_len),
                                 g.ctypes.data, _ptr(g_off), _ptr(g_cap), _ptr(g_len), _ptr(st))
        return g, g_off, g_len, st

    def batch_upload(self, limbs, u_off, u_len, v_off, v_len):
        self._batch_layout = (len(u_off),) + result_layout(u_len, v_len)
        _check(self._lib.mgcd_batch_upload(self._h, len(u_off), _ptr(limbs), _ptr(u_off), _ptr(u_len),
                                           _ptr(v_off), _ptr(v_len)))

    def batch_run(self):
        _check(self._lib.mgcd_batch_run(self._h))

    def batch_sync(self):
        _check(self._lib.mgcd_batch_sync(self._h))

    def batch_download(self):
        n, g_off, g_cap, tot = self._batch_layout
        g = np.zeros(max(tot, 1), dtype=np.uint32)
        g_len = np.zeros(n, dtype=np.uint32)
        st = np.zeros(n, dtype=np.int32)
        self._lib.mgcd_batch_download(self._h, g.ctypes.data, _ptr(g_off), _ptr(g_cap), _ptr(g_len), _ptr(st))
        return g, g_off, g_len, st

    def set_nq_scale(self, scale):
        """Fraction of the reference moduli count batches use (results are certified)."""
        _check(self._lib.mgcd_set_nq_scale(self._h, float(scale)))

    def set_growth(self, start, step_permille=50):
        """Moduli grown on demand in batches (mgcd_set_growth; start 0 turns it off)."""
        _check(self._lib.mgcd_set_growth(self._h, float(start), int(step_permille)))

    def growth(self):
        st, pm = ctypes.c_float(), ctypes.c_uint()
        _check(self._lib.mgcd_get_growth(self._h, ctypes.byref(st), ctypes.byref(pm)))
        return st.value, pm.value

    def batch_pair_digits(self, i):
        """Digits [(modulus, value), ...] of pair i of the last batch and its final moduli count."""
        n, nqf = ctypes.c_size_t(), ctypes.c_uint32()
        rc = self._lib.mgcd_batch_pair_digits(self._h, i, None, 0, ctypes.byref(n), ctypes.byref(nqf))
        if rc not in (MGCD_OK, MGCD_ERR_CAPACITY):
            _check(rc)
        d = np.zeros(max(1, n.value), dtype=[("modulus", "<u4"), ("value", "<i4")])
        _check(self._lib.mgcd_batch_pair_digits(self._h, i, d.ctypes.data, n.value, ctypes.byref(n),
                                                ctypes.byref(nqf)))
        return [(int(m), int(x)) for m, x in d[: n.value]], int(nqf.value)

    def set_size_class(self, cls, threads, k, nq_scale):
        """Launch configuration of size class cls (0: <= 1024 moduli, 1: <= 4096,
        2: <= 16384, 3: larger, one thread-block cluster per pair)."""
        _check(self._lib.mgcd_set_size_class(self._h, int(cls), int(threads), int(k), float(nq_scale)))

    def set_cluster_size(self, ctas):
        """CTAs per cluster of size class 3."""
        _check(self._lib.mgcd_set_cluster_size(self._h, int(ctas)))

    def get_cluster_size(self):
        n = ctypes.c_int()
        _check(self._lib.mgcd_get_cluster_size(self._h, ctypes.byref(n)))
        return n.value

    def certify_inverse(self):
        """Exhaustive end-point certification of the inverse's quotient steps on this GPU:
        {"checked", "failures", "first_failure"}."""
        n, f, a, b = ctypes.c_uint64(), ctypes.c_uint64(), ctypes.c_uint32(), ctypes.c_uint32()
        _check(self._lib.mgcd_certify_inverse(self._h, ctypes.byref(n), ctypes.byref(f), ctypes.byref(a),
                                              ctypes.byref(b)))
        return {"checked": n.value, "failures": f.value,
                "first_failure": (a.value, b.value) if f.value else None}

    def load_tuning(self, path):
        """Applies a tuning table (mgcd_load_tuning)."""
        if not os.path.exists(path):
            raise OSError("no tuning table at %s" % path)
        _check(self._lib.mgcd_load_tuning(self._h, os.fsencode(path)))

    def save_tuning(self, path):
        _check(self._lib.mgcd_save_tuning(self._h, os.fsencode(path)))

    def set_class_cluster(self, cls, ctas):
        """CTAs per cluster for size class cls (0: one CTA per pair, classes 0-2 only)."""
        _check(self._lib.mgcd_set_class_cluster(self._h, int(cls), int(ctas)))

    def get_class_cluster(self, cls):
        n = ctypes.c_int()
        _check(self._lib.mgcd_get_class_cluster(self._h, int(cls), ctypes.byref(n)))
        return n.value

    def batch_use_graph(self, enable=True):
        """Record each upload's GPU work into a CUDA graph and replay it on every run."""
        _check(self._lib.mgcd_batch_use_graph(self._h, 1 if enable else 0))

    def set_single_pair_policy(self, policy):
        """0: cluster / grid (default); 1: the reference's launch shape (grid of 256-thread CTAs)."""
        _check(self._lib.mgcd_set_single_pair_policy(self._h, int(policy)))

    def set_wait_timeout_ms(self, ms):
        _check(self._lib.mgcd_set_wait_timeout_ms(self._h, int(ms)))

    def test_withhold_cta(self, cta):
        """Test hook: CTA `cta` of grid-mode pairs never publishes (-1: off)."""
        _check(self._lib.mgcd_test_withhold_cta(self._h, int(cta)))

    def test_fail_staging(self, cta):
        """Test hook: CTA `cta` of later kernels reports an operand-staging failure (-1: off)."""
        _check(self._lib.mgcd_test_fail_staging(self._h, int(cta)))

    def test_force_moduli(self, nq):
        """Test hook: every pair uses exactly nq moduli, no rerun (0: reference count)."""
        _check(self._lib.mgcd_test_force_moduli(self._h, int(nq)))

    def get_size_class(self, cls):
        t, k, s = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
        _check(self._lib.mgcd_get_size_class(self._h, int(cls), ctypes.byref(t), ctypes.byref(k), ctypes.byref(s)))
        return t.value, k.value, s.value

    def batch_kernel_stats(self):
        """[(size class, pairs, ms)] of the last run's kernels."""
        out = []
        i = 0
        while True:
            c, n, ms = ctypes.c_int(), ctypes.c_int(), ctypes.c_float()
            if self._lib.mgcd_batch_kernel_stats(self._h, i, ctypes.byref(c), ctypes.byref(n), ctypes.byref(ms)) != 0:
                return out
            out.append((c.value, n.value, ms.value))
            i += 1

    def batch_kernel_work(self, i):
        """Cost-model work of kernel i of the last downloaded batch."""
        r, e, m, b = (ctypes.c_double() for _ in range(4))
        _check(self._lib.mgcd_batch_kernel_work(self._h, int(i), ctypes.byref(r), ctypes.byref(e), ctypes.byref(m),
                                                ctypes.byref(b)))
        ab = ctypes.c_double()
        _check(self._lib.mgcd_batch_alg_bytes(self._h, ctypes.byref(ab)))
        return {"residue_steps": r.value, "euclid_updates": e.value, "recovery_updates": m.value,
                "operand_bytes": b.value, "algorithmic_bytes": ab.value}

    def batch_retried(self):
        n = ctypes.c_int()
        _check(self._lib.mgcd_batch_retried(self._h, ctypes.byref(n)))
        return n.value

    def batch_launches(self):
        n = ctypes.c_int()
        _check(self._lib.mgcd_batch_launches(self._h, ctypes.byref(n)))
        return n.value

    def batch_elapsed_ms(self):
        """(run_ms, dominant_kernel_ms, dominant_threads) of the last run, by CUDA events."""
        r, d, t = ctypes.c_float(), ctypes.c_float(), ctypes.c_int()
        _check(self._lib.mgcd_batch_elapsed_ms(self._h, ctypes.byref(r), ctypes.byref(d), ctypes.byref(t)))
        return r.value, d.value, t.value

    def batch_transfer_bytes(self):
        h, d = ctypes.c_uint64(), ctypes.c_uint64()
        _check(self._lib.mgcd_batch_transfer_bytes(self._h, ctypes.byref(h), ctypes.byref(d)))
        return h.value, d.value

    def int_peak(self):
        """Measured 32-bit IMAD throughput of the GPU (instructions/s)."""
        x = ctypes.c_double()
        _check(self._lib.mgcd_int_peak(self._h, ctypes.byref(x)))
        return x.value

    def set_cta_trace(self, enable=True):
        """Record per-CTA occupancy of the batched kernels in later runs."""
        _check(self._lib.mgcd_set_cta_trace(self._h, int(bool(enable))))

    def batch_cta_trace(self):
        """The last run's per-CTA records (structured array, CTA_RECORD)."""
        n = ctypes.c_size_t()
        _check(self._lib.mgcd_batch_cta_trace(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=CTA_RECORD)
        if n.value:
            _check(self._lib.mgcd_batch_cta_trace(self._h, out.ctypes.data, n.value, ctypes.byref(n)))
        return out

    def batch_work(self):
        r, e, m, b = (ctypes.c_double() for _ in range(4))
        _check(self._lib.mgcd_batch_work(self._h, ctypes.byref(r), ctypes.byref(e), ctypes.byref(m),
                                         ctypes.byref(b)))
        ab = ctypes.c_double()
        _check(self._lib.mgcd_batch_alg_bytes(self._h, ctypes.byref(ab)))
        return {"residue_steps": r.value, "euclid_updates": e.value, "recovery_updates": m.value,
                "operand_bytes": b.value, "algorithmic_bytes": ab.value}


CTA_RECORD = np.dtype([("size_class", "<i4"), ("sm", "<u4"), ("pairs", "<u4"), ("ran", "<i4"),
                       ("t_start_ms", "<f8"), ("t_end_ms", "<f8"), ("cycles_setup", "<u8"),
                       ("cycles_update", "<u8"), ("cycles_pivot", "<u8"), ("cycles_finish", "<u8"),
                       ("iterations", "<u8"), ("rounds", "<u8"), ("cycles_replay", "<u8"),
                       ("update_rounds", "<u8"), ("rounds_with_inverse", "<u8"), ("finite_slot_updates", "<u8"),
                       ("cycles_layout", "<u8"), ("cycles_grow", "<u8"), ("grow_steps", "<u8")])


class Server:
    """Request server on a Device (mgcd_serve_*): continuous batching of single requests
    under an HBM admission budget.  The Device's own calls are refused while it runs."""

    def __init__(self, device, budget_bytes=8 << 30):
        self._lib = device._lib
        self.device = device
        h = ctypes.c_void_p()
        _check(self._lib.mgcd_serve_start(device._h, int(budget_bytes), ctypes.byref(h)))
        self._h = h

    def close(self):
        if getattr(self, "_h", None):
            self._lib.mgcd_serve_stop(self._h)
            self._h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *exc):
        self.close()

    def set_continuous(self, enable=True):
        """Continuous lanes for size classes 0-1 (default on) or waves for every request."""
        _check(self._lib.mgcd_serve_set_continuous(self._h, int(bool(enable))))

    def submit(self, u, v):
        a, b = to_limbs(u), to_limbs(v)
        t = ctypes.c_uint64()
        _check(self._lib.mgcd_serve_submit(self._h, _ptr(a), len(a), _ptr(b), len(b), ctypes.byref(t)))
        return t.value

    def poll(self, ticket):
        d = ctypes.c_int()
        _check(self._lib.mgcd_serve_poll(self._h, int(ticket), ctypes.byref(d)))
        return bool(d.value)

    def take(self, ticket, cap, timeout_ms=0):
        """(gcd, latency_s) of a ticket; cap >= the result's limb count."""
        g = np.zeros(max(int(cap), 1), dtype=np.uint32)
        n, lat = ctypes.c_size_t(), ctypes.c_double()
        _check(self._lib.mgcd_serve_take(self._h, int(ticket), int(timeout_ms), g.ctypes.data, len(g),
                                         ctypes.byref(n), ctypes.byref(lat)))
        return from_limbs(g[: n.value]), lat.value

    def gcd(self, u, v):
        """One request, submitted and waited for."""
        t = self.submit(u, v)
        return self.take(t, max(len(to_limbs(u)), len(to_limbs(v))) + 1)[0]

    def replay_packed(self, limbs, u_off, u_len, v_off, v_len, arrival_s):
        """Open-loop load (mgcd_serve_replay): (g, g_off, g_len, status, latency_s, makespan_s)."""
        n = len(u_off)
        g_off, g_cap, tot = result_layout(u_len, v_len)
        g = np.zeros(max(tot, 1), dtype=np.uint32)
        g_len = np.zeros(n, dtype=np.uint32)
        st = np.zeros(n, dtype=np.int32)
        lat = np.zeros(n, dtype=np.float64)
        arr = np.ascontiguousarray(arrival_s, dtype=np.float64)
        mk = ctypes.c_double()
        self._lib.mgcd_serve_replay(self._h, n, _ptr(limbs), _ptr(u_off), _ptr(u_len), _ptr(v_off), _ptr(v_len),
                                    _ptr(arr), g.ctypes.data, _ptr(g_off), _ptr(g_cap), _ptr(g_len), _ptr(st),
                                    _ptr(lat), ctypes.byref(mk))
        return g, g_off, g_len, st, lat, mk.value

    def replay(self, us, vs, arrival_s):
        """[gcd] per request, statuses, latencies (s) and the makespan (s)."""
        g, g_off, g_len, st, lat, mk = self.replay_packed(*pack_pairs(us, vs), arrival_s)
        res = [from_limbs(g[int(o): int(o) + int(n)]) for o, n in zip(g_off, g_len)]
        return res, st, lat, mk

    WAVE_TRACE = np.dtype([("lane", "<i4"), ("requests", "<u4"), ("t_admit", "<f8"), ("t_launched", "<f8"),
                           ("t_gpu_done", "<f8"), ("t_answered", "<f8")])

    def trace(self):
        """Per-wave records (mgcd_serve_trace) as a numpy structured array."""
        n = ctypes.c_size_t()
        _check(self._lib.mgcd_serve_trace(self._h, None, 0, ctypes.byref(n)))
        out = np.zeros(n.value, dtype=self.WAVE_TRACE)
        _check(self._lib.mgcd_serve_trace(self._h, out.ctypes.data if n.value else None, n.value, ctypes.byref(n)))
        return out[: n.value]

    def stats(self):
        w, l, p, c = (ctypes.c_uint64() for _ in range(4))
        _check(self._lib.mgcd_serve_stats(self._h, ctypes.byref(w), ctypes.byref(l), ctypes.byref(p),
                                          ctypes.byref(c)))
        return {"waves": w.value, "launches": l.value, "peak_admitted_bytes": p.value, "completed": c.value}


def build(verbose=False):
    """Compiles libmodgcd.so / libGmpCuda.so in-tree (nvcc for sm_103a)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("_mgcd_build", os.path.join(HERE, "build.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod.build(verbose=verbose)
