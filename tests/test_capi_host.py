"""Host-side checks of the boundary (no GPU needed): the C ABI library loads and exports
every symbol include/modgcd.h declares; the product's moduli table and moduli count agree
with the oracle and the reference; the C++ drop-in compiles against the reference's own
test driver; error behaviour without a device."""
import ctypes
import math
import os
import re
import subprocess

import numpy as np
import pytest

from conftest import ROOT

HEADER = os.path.join(ROOT, "include", "modgcd.h")
# the reference's sources as installed by `make -C baseline install`
REFERENCE = os.path.join(ROOT, "baseline", "_ref", "src")


def declared_functions():
    src = open(HEADER).read()
    src = re.sub(r"/\*.*?\*/", "", src, flags=re.S)
    return sorted(set(re.findall(r"\b(mgcd_\w+)\s*\(", src)))


def test_library_exports_every_declared_symbol(mgcd):
    lib = ctypes.CDLL(mgcd.LIB_PATH)
    names = declared_functions()
    assert len(names) >= 19
    missing = [n for n in names if not hasattr(lib, n)]
    assert not missing, missing
    assert set(names) == set(mgcd.SIGNATURES), "Python binding out of sync with modgcd.h"


def test_dropin_library_exports(mgcd):
    lib = ctypes.CDLL(os.path.join(mgcd.LIB_DIR, "libGmpCuda.so"))
    for sym in ("_ZN7GmpCuda13GmpCudaDevice9setDeviceEi", "_ZN7GmpCuda13GmpCudaDeviceC1Ev",
                "_ZN7GmpCuda13GmpCudaDeviceD1Ev", "_ZN7GmpCuda13GmpCudaDevice3gcdEP12__mpz_structS2_S2_",
                "_ZN7GmpCuda6moduliE", "_ZN7GmpCuda13moduliInverseE"):
        assert hasattr(lib, sym), sym


def test_product_moduli_match_oracle(mgcd, oracle):
    for L, n in ((32, 131072), (27, 20000), (22, 97358)):
        a = mgcd.gen_moduli(L, n)
        b = oracle.gen_moduli(L, n)
        assert np.array_equal(a, b), L
    for L in (22, 27, 32):
        for bits in (1, 2, 100, 1024, 10240, 65536, 1 << 20, 1300000):
            assert mgcd.moduli_needed(bits, L) == oracle.num_moduli_needed(bits, L)


def test_createModuli_tool_matches_reference_format(mgcd):
    exe = os.path.join(mgcd.LIB_DIR, "createModuli")
    out = subprocess.run([exe, "32", "65536"], capture_output=True, text=True, check=True)
    lines = out.stdout.split("\n")
    assert lines[0] == "//  AUTOMATICALLY GENERATED by createModuli: do not edit"
    assert "const uint32_t GmpCuda::moduli[] = " in lines
    body = [int(x) for x in re.findall(r"^\t(\d+),$", out.stdout, re.M)]
    assert len(body) == 65536 and body[:2] == [4294967291, 4294967279]
    assert out.stderr.strip() == "65536 moduli were generated."
    short = subprocess.run([exe, "22", "200000"], capture_output=True, text=True)
    assert short.returncode == 2          # too few usable moduli (createModuli.cpp:171-178)
    inv = subprocess.run([exe, "32", "4", "--inverses"], capture_output=True, text=True, check=True).stdout
    js = [int(x) for x in re.findall(r"^\t(\d+)ull,$", inv, re.M)]
    qs = [int(x) for x in re.findall(r"^\t(\d+),$", inv, re.M)]
    assert js == [(1 << 95) // q + 1 for q in qs]


def test_no_device_errors(mgcd):
    if mgcd.device_count() > 0:
        pytest.skip("a GPU is present")
    with pytest.raises(mgcd.GcdError) as e:
        mgcd.Device.set_device(0)
    assert str(e.value) == "Invalid device number."
    with pytest.raises(mgcd.GcdError) as e:
        mgcd.Device(0)
    assert e.value.status == mgcd.MGCD_ERR_NO_DEVICE
    assert mgcd.status_string(6) == "Ran out of moduli in the reduction loop."
    assert mgcd.status_string(4) == "Not enough moduli available for given input."


def test_batch_layout_helpers(mgcd):
    us = [0, 1, 2 ** 100 + 5, 12345678901234567890]
    vs = [7, 0, 3, 2 ** 64]
    limbs, uo, ul, vo, vl = mgcd.pack_pairs(us, vs)
    for i, (u, v) in enumerate(zip(us, vs)):
        assert mgcd.from_limbs(limbs[int(uo[i]): int(uo[i]) + int(ul[i])]) == u
        assert mgcd.from_limbs(limbs[int(vo[i]): int(vo[i]) + int(vl[i])]) == v
    off, cap, tot = mgcd.result_layout(ul, vl)
    assert tot == int(cap.sum()) and all(cap >= 1)


@pytest.mark.skipif(not os.path.isfile(os.path.join(REFERENCE, "testmodgcd.cpp")),
                    reason="reference sources not installed")
def test_reference_testmodgcd_compiles_against_dropin(mgcd, tmp_path):
    """The reference's own test driver compiles and links unchanged against GmpCuda.h."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("b", os.path.join(ROOT, "modgcd-onegpu_gb300", "build.py"))
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    exe = str(tmp_path / "testmodgcd")
    cmd = ["g++", "--std=c++14", "-O2", "-I" + os.path.join(ROOT, "include")] + b.gmp_include_flags() + \
          [os.path.join(REFERENCE, "testmodgcd.cpp"), "-o", exe, "-L" + mgcd.LIB_DIR, "-lGmpCuda", "-lmodgcd",
           "-Wl,-rpath," + mgcd.LIB_DIR, "-l:libgmp.so.10"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    assert os.path.exists(exe)


def test_tuning_tables_width_choice_and_traffic_record(mgcd):
    """The committed tuning artifacts the benchmark reads: one table per modulus width in the
    loader's format (class threads k nq_scale cluster_ctas, an optional 'grow start permille'
    line, '#' comments), the width choice, and an ncu traffic figure for every width the
    batched benchmark can run."""
    import json
    tdir = os.path.join(os.path.dirname(mgcd.__file__), "tuning")
    for L in (22, 27, 32):
        rows = [ln.split() for ln in open(os.path.join(tdir, "gb300_L%d.txt" % L))
                if ln.strip() and not ln.lstrip().startswith("#")]
        grow = [r for r in rows if r[0] == "grow"]
        rows = [r for r in rows if r[0] != "grow"]
        assert len(grow) <= 1
        for _, start, permille in grow:
            assert 0.1 <= float(start) <= 1.0 and 10 <= int(permille) <= 500
        assert sorted(int(r[0]) for r in rows) == [0, 1, 2, 3]
        for cls, threads, k, scale, cs in rows:
            assert int(threads) in (256, 512, 1024) and int(k) in (1, 2, 4, 8)
            assert 0.5 <= float(scale) <= 1.0 and int(cs) in (0, 2, 4, 8, 16)
    assert mgcd.tuned_width() in (22, 27, 32)
    root = os.path.dirname(os.path.dirname(os.path.abspath(mgcd.__file__)))
    traffic = json.load(open(os.path.join(root, "profiles", "ncu_traffic.json")))["by_modulus_bits"]
    assert str(mgcd.tuned_width()) in traffic and "32" in traffic
    for rec in traffic.values():
        assert abs(rec["bytes_per_pair"] - rec["dram_bytes"] / rec["pairs"]) < 1
        assert os.path.exists(os.path.join(root, "profiles", rec["source"]))
