"""Generates the golden fixtures in this directory (run here, where the reference sources exist).

Inputs come from the reference itself: its test driver, built without a GPU
(``make -C oracle ref`` -> ``oracle/_ref/testmodgcd-nogpu``), writes the pairs it tests to
``tests/<bits>-<gcd_bits>`` as base-62 ``mpz_out_str`` lines, two per pair, drawn from
``gmp_randinit_mt`` with its default seed (testmodgcd.cpp:173-259).  Those files are copied
here verbatim (optionally cut to the first few pairs) as ``ref_<bits>-<gcd_bits>.txt``.

Expected outputs come from GMP ``mpz_gcd`` -- the reference's own oracle
(testmodgcd.cpp:441) -- through ``oracle/libcpugmp.so``; they are cross-checked against
Python's exact gcd.  ``golden.json`` also records, per pair, what the oracle's restatement
of the kernel does (moduli count, reduction iterations, digit count, status) so that a
change of the restatement shows up as a fixture mismatch.

The moduli fixture ``ref_moduli_L32.txt`` is the head and tail of the reference's
createModuli output, plus a checksum of all 65,536 entries.

``config1_seed1.txt`` is the single-pair benchmark configuration's pair (g 2048-bit odd,
a and b 8192-bit coprime, GMP Mersenne Twister seeded with 1; workloads.single_pair) in the
same two-line base-62 format, followed by its gcd from mpz_gcd.  The generator it comes
from reproduces the reference driver's files above draw for draw (workloads.reference_pairs,
checked by tests/test_workloads.py), so the fixture pins the configuration's inputs.

Usage:  python tests/golden/make_golden.py [--config1-only]
"""
import hashlib
import json
import math
import os
import re
import shutil
import subprocess
import sys
import tempfile

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
import pyoracle as po  # noqa: E402

# (bits, gcd_bits, pairs kept)
CASES = [(64, 1, 10), (256, 64, 10), (1024, 1, 10), (4096, 1024, 10), (10240, 2048, 10),
         (16384, 1, 4), (16384, 4096, 4), (65536, 16384, 2)]

B62 = "0123456789ABCDEFGHIJKLMNOPQRSTUVWXYZabcdefghijklmnopqrstuvwxyz"


def parse_b62(s: str) -> int:
    """GMP's base-62 digits: 0-9, A-Z (10-35), a-z (36-61)."""
    x = 0
    for ch in s.strip():
        x = x * 62 + B62.index(ch)
    return x


def to_b62(x: int) -> str:
    s = []
    while x:
        x, r = divmod(x, 62)
        s.append(B62[r])
    return "".join(reversed(s)) or "0"


def write_config1():
    import importlib
    sys.path.insert(0, ROOT)
    wl = importlib.import_module("modgcd-onegpu_gb300.workloads")
    u, v = wl.single_pair(seed=1)
    a, b = po.to_limbs(u), po.to_limbs(v)
    _, g, goff, glen = po.cpu_gmp_gcd_batch(np.concatenate([a, b]), [0], [len(a)], [len(a)], [len(b)], 1)
    gm = po.from_limbs(g[int(goff[0]): int(goff[0]) + int(glen[0])])
    assert gm == math.gcd(u, v)
    with open(os.path.join(HERE, "config1_seed1.txt"), "w") as f:
        f.write(to_b62(u) + "\n" + to_b62(v) + "\n" + to_b62(gm) + "\n")


def main():
    write_config1()
    if "--config1-only" in sys.argv:
        return
    oracle = os.path.join(ROOT, "oracle")
    subprocess.run(["make", "-s", "-C", oracle, "all", "ref"], check=True)
    driver = os.path.join(oracle, "_ref", "testmodgcd-nogpu")
    creat = os.path.join(oracle, "_ref", "createModuli")
    golden = {"generator": "reference testmodgcd-nogpu (gmp_randinit_mt default seed)",
              "gmp": po.gmp_version(), "cases": []}
    mod32 = po.gen_moduli(32, 131072)
    for bits, gbits, keep in CASES:
        with tempfile.TemporaryDirectory() as tmp:
            subprocess.run([driver, str(bits), str(gbits)], cwd=tmp, check=True, stdout=subprocess.DEVNULL)
            lines = open(os.path.join(tmp, "tests", f"{bits}-{gbits}")).read().split("\n")
        lines = [ln for ln in lines if ln.strip()][: 2 * keep]
        name = f"ref_{bits}-{gbits}.txt"
        with open(os.path.join(HERE, name), "w") as f:
            f.write("\n".join(lines) + "\n")
        us = [parse_b62(lines[2 * i]) for i in range(keep)]
        vs = [parse_b62(lines[2 * i + 1]) for i in range(keep)]
        packed, uo, ul, vo, vl = [], [], [], [], []
        off = 0
        for u, v in zip(us, vs):
            a, b = po.to_limbs(u), po.to_limbs(v)
            uo.append(off); ul.append(len(a)); packed.append(a); off += len(a)
            vo.append(off); vl.append(len(b)); packed.append(b); off += len(b)
        _, g, goff, glen = po.cpu_gmp_gcd_batch(np.concatenate(packed), uo, ul, vo, vl, 1)
        pairs = []
        for i, (u, v) in enumerate(zip(us, vs)):
            gm = po.from_limbs(g[int(goff[i]): int(goff[i]) + int(glen[i])])
            assert gm == math.gcd(u, v)
            uu, vv = (u, v) if u >= v else (v, u)
            nq = po.num_moduli_needed(uu.bit_length(), 32)
            st, dig, tr, it = po.modgcd(uu, vv, 32, mod32, nq)
            if st == po.ORC_OK:
                assert po.mixed_radix_to_int(dig) == gm
            pairs.append({"gcd_hex": format(gm, "x"), "nq": nq, "status": st, "iters": it,
                          "digits": len(dig),
                          "trace_sha1": hashlib.sha1(repr(tr).encode()).hexdigest(),
                          "digits_sha1": hashlib.sha1(repr(dig).encode()).hexdigest()})
        golden["cases"].append({"file": name, "bits": bits, "gcd_bits": gbits, "pairs": pairs})
        print(name, [p["iters"] for p in pairs])
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(golden, f, indent=1)

    # moduli table from the reference's generator
    with tempfile.TemporaryDirectory() as tmp:
        out = subprocess.run([creat], cwd=tmp, check=True, capture_output=True, text=True).stdout
    ref = np.array([int(x) for x in re.findall(r"^\t(\d+),", out, re.M)], dtype=np.uint32)
    assert len(ref) == 65536
    with open(os.path.join(HERE, "ref_moduli_L32.txt"), "w") as f:
        f.write("# reference createModuli (L=32, W=64): count, sha1 of the little-endian uint32 array,\n")
        f.write("# then the first 64 and last 64 entries\n")
        f.write(f"count {len(ref)}\n")
        f.write(f"sha1 {hashlib.sha1(ref.astype('<u4').tobytes()).hexdigest()}\n")
        f.write("head " + " ".join(map(str, ref[:64])) + "\n")
        f.write("tail " + " ".join(map(str, ref[-64:])) + "\n")
    shutil.rmtree(os.path.join(ROOT, "tests", "golden", "__pycache__"), ignore_errors=True)


if __name__ == "__main__":
    main()
