"""The allocation-free entry point (mgcd_gcd_digits_noalloc) against the regular one.

mgcd_gcd_digits_noalloc serves callers that cannot allocate device memory when they need
a gcd (real-time or callback contexts that must not wait on the allocator, applications
whose device memory is budgeted by their own pools): they pass device buffers for the
operands and results, and the library works in one static device array instead of
allocating.  This test owns its buffers (allocated here, through torch), calls the entry
point through the C ABI twice in a row on different pairs -- the second call reuses the
scratch array the first call left behind -- and requires the digits, count and status to
equal what the regular entry point (mgcd_gcd_digits) returns.  It also runs a pair at the
4,096-moduli limit, where the history and the initial residues fill the static array,
and checks that a pair over the limit is refused before any launch.
"""
import math
import random

import numpy as np
import pytest

pytestmark = pytest.mark.gpu


def _pairs():
    rng = random.Random(2024)
    g = rng.getrandbits(2048) | (1 << 2047) | 1
    first = (g * (rng.getrandbits(8192) | (1 << 8191)), g * (rng.getrandbits(8000) | 1))
    h = rng.getrandbits(600) | 1
    second = (h * (rng.getrandbits(30000) | (1 << 29999)), h * (rng.getrandbits(20000) | 1))
    return [first, second]


def _call_noalloc(mgcd, torch, u, v):
    lib = mgcd.load()
    a, b = mgcd.to_limbs(u), mgcd.to_limbs(v)
    limbs = torch.from_numpy(np.concatenate([a, b]).view(np.int32)).cuda()
    cap = mgcd.moduli_needed(32 * max(len(a), len(b)), 32)
    d_dig = torch.zeros(2 * cap, dtype=torch.int32, device="cuda")
    d_cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    d_st = torch.full((1,), -1, dtype=torch.int32, device="cuda")
    stream = torch.cuda.current_stream()
    rc = lib.mgcd_gcd_digits_noalloc(limbs.data_ptr(), len(a), len(b), d_dig.data_ptr(), cap, d_cnt.data_ptr(),
                                     d_st.data_ptr(), stream.cuda_stream)
    assert rc == 0, mgcd.status_string(rc)
    torch.cuda.synchronize()
    n = int(d_cnt.item())
    raw = d_dig[: 2 * n].cpu().numpy()
    digits = [(int(np.uint32(raw[2 * i].item() & 0xFFFFFFFF)), int(raw[2 * i + 1])) for i in range(n)]
    return int(d_st.item()), digits


def test_noalloc_matches_regular_entry_point(mgcd):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    with mgcd.Device(0, 32) as dev:
        for u, v in _pairs():                      # two calls in a row, shared scratch
            expected = dev.gcd_digits(u, v)
            status, digits = _call_noalloc(mgcd, torch, u, v)
            assert status == 0
            assert digits == expected
        u, v = _pairs()[0]
        status, digits = _call_noalloc(mgcd, torch, v, u)   # operands in the other order
        assert status == 0 and digits == dev.gcd_digits(u, v)
        import pyoracle
        assert pyoracle.mixed_radix_to_int(digits) == math.gcd(u, v)


def test_noalloc_at_the_moduli_limit(mgcd):
    """Operands that need exactly 4,096 moduli (37,000-38,600 bits): the scratch array is
    used to its end; two such calls in a row, each equal to the regular entry point."""
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    rng = random.Random(2025)
    with mgcd.Device(0, 32) as dev:
        for ubits, vbits, gbits in [(38600, 38000, 9000), (37000, 36990, 1)]:
            assert mgcd.moduli_needed(32 * ((ubits + 31) // 32), 32) == 4096
            g = rng.getrandbits(gbits) | (1 << (gbits - 1)) | 1
            u = g * (rng.getrandbits(ubits - gbits) | (1 << (ubits - gbits - 1)))
            v = g * (rng.getrandbits(vbits - gbits) | 1)
            status, digits = _call_noalloc(mgcd, torch, u, v)
            assert status == 0
            assert digits == dev.gcd_digits(u, v)


def test_noalloc_rejects_sizes_over_limit(mgcd):
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    lib = mgcd.load()
    x = torch.ones(2600, dtype=torch.int32, device="cuda")   # 41,600-bit operands need > 4,096 moduli
    out = torch.zeros(2 * 8192, dtype=torch.int32, device="cuda")
    cnt = torch.zeros(1, dtype=torch.int32, device="cuda")
    st = torch.full((1,), 12345, dtype=torch.int32, device="cuda")
    rc = lib.mgcd_gcd_digits_noalloc(x.data_ptr(), 1300, 1300, out.data_ptr(), 8192, cnt.data_ptr(), st.data_ptr(),
                                     torch.cuda.current_stream().cuda_stream)
    assert mgcd.STATUS_NAMES[rc] == "MGCD_ERR_NOT_ENOUGH_MODULI"
    assert mgcd.status_string(rc) == "Not enough moduli available for given input."
    torch.cuda.synchronize()
    assert int(st.item()) == 12345                 # nothing was launched
