#!/usr/bin/env python
"""Autotuner of the batched path: picks, per size class, the launch configuration that
gives the shortest device time for that class's pairs, and writes the tuning table that
mgcd_load_tuning reads.

Size classes (by the reference's moduli count of the pair): 0 = <= 1,024 moduli, 1 =
<= 4,096, 2 = <= 16,384 (one CTA per pair), 3 = larger (one thread-block cluster per pair).
Candidates: CTA size 256/512/1024, pairs per CTA in lockstep k = 1/2/4/8 (k = 8 needs
512 threads), fraction of the reference moduli count 1.0 ... 0.7
(results stay exact: uncertified pairs are rerun, and the rerun is part of the timed run),
and for classes 0-2 also clusters of 2 or 4 CTAs per k pairs (the longest pairs of a batch
bound its time when each runs on one SM); for class 3 the CTA size, the pairs per cluster
(1/2/4) and the cluster size (4/8/16 CTAs).  The classes of a batch run concurrently and
share the SMs, so classes 0-2 are
tuned by coordinate descent on the whole mixed
1k-64k-bit batch (largest class first, the others held at their current best); class 3 is
timed alone on 300k-bit pairs.  Every time is the median of `reps` runs and every result
is checked against Python's gcd.

  python modgcd-onegpu_gb300/tune.py [--out PATH] [--log PATH] [--L 32]
  python modgcd-onegpu_gb300/tune.py --refine --L 27 --seed 11   (finer moduli fraction)
"""
import argparse
import importlib
import json
import math
import os
import statistics
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.dirname(HERE))

mg = importlib.import_module("modgcd-onegpu_gb300")
wl = importlib.import_module("modgcd-onegpu_gb300.workloads")

SCALES = (1.0, 0.9, 0.8, 0.7)


def class_of(u, v, L):
    nq = mg.moduli_needed(max(u.bit_length(), v.bit_length()), L)
    return 0 if nq <= 1024 else 1 if nq <= 4096 else 2 if nq <= 16384 else 3


def time_config(dev, packed, exp, reps):
    dev.batch_upload(*packed)
    ms = []
    for _ in range(reps + 1):
        dev.batch_run()
        dev.batch_sync()
        ms.append(dev.batch_elapsed_ms()[0])
    g, go, gn, st = dev.batch_download()
    got = [mg.from_limbs(g[int(o): int(o) + int(n)]) for o, n in zip(go, gn)]
    if not (st == 0).all() or got != exp:
        raise RuntimeError("tuning run gave a wrong or failed result")
    return statistics.median(ms[1:])


def compare_widths(args):
    """Times the whole mixed batch at each modulus width with that width's tuning table and
    writes the fastest width to tuning/gb300_width.txt (read by mg.tuned_width())."""
    us, vs, _ = wl.mixed_batch(args.pairs, seed=args.seed)
    packed = mg.pack_pairs(us, vs)
    exp = [math.gcd(u, v) for u, v in zip(us, vs)]
    res = {}
    for L in (32, 27, 22):
        with mg.Device(0, L) as dev:
            dev.load_tuning(os.path.join(HERE, "tuning", "gb300_L%d.txt" % L))
            res[L] = time_config(dev, packed, exp, args.reps)
            print(json.dumps({"L": L, "ms": res[L]}), flush=True)
    best = min(res, key=res.get)
    out = args.out or os.path.join(HERE, "tuning", "gb300_width.txt")
    with open(out, "w") as f:
        f.write("%d\n# modulus width with the fastest whole mixed batch (%d pairs, seed %d): %s\n" %
                (best, args.pairs, args.seed, ", ".join("L=%d %.1f ms" % (L, res[L]) for L in sorted(res))))
    print(open(out).read())


REFINE_STEPS = (-0.08, -0.06, -0.04, -0.02, 0.0, 0.02, 0.04, 0.06, 0.08)


def refine(args):
    """Second pass over a width's table: the moduli fraction of classes 2, 1, 0 on a finer
    grid (steps of 0.02 around the table's value), every other setting held, on the whole
    mixed batch.  The fraction trades work per iteration against reruns, and the time has a
    sharp edge below the best value, which the first pass's 0.1 grid brackets only loosely."""
    us, vs, _ = wl.mixed_batch(args.pairs, seed=args.seed)
    packed = mg.pack_pairs(us, vs)
    exp = [math.gcd(u, v) for u, v in zip(us, vs)]
    path = os.path.join(HERE, "tuning", "gb300_L%d.txt" % args.L)
    log, best = [], {}
    with mg.Device(0, args.L) as dev:
        dev.load_tuning(path)
        for c in (2, 1, 0):
            t, k, s0 = dev.get_size_class(c)
            for d in REFINE_STEPS:
                s = round(s0 + d, 3)
                if not 0.5 <= s <= 1.0:
                    continue
                dev.set_size_class(c, t, k, s)
                ms = time_config(dev, packed, exp, args.reps)
                log.append({"class": c, "threads": t, "k": k, "nq_scale": s, "cluster": dev.get_class_cluster(c),
                            "ms": ms, "retried": dev.batch_retried()})
                print(json.dumps(log[-1]), flush=True)
                if c not in best or ms < best[c][0]:
                    best[c] = (ms, s)
            dev.set_size_class(c, t, k, best[c][1])
        out = args.out or path
        dev.save_tuning(out)
    if args.log:
        with open(args.log, "w") as f:
            json.dump({"best": {str(c): b for c, b in best.items()}, "runs": log, "seed": args.seed}, f, indent=1)
    print(open(out).read())


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--L", type=int, default=32)
    ap.add_argument("--compare-widths", action="store_true",
                    help="time the mixed batch at every width with its table; write tuning/gb300_width.txt")
    ap.add_argument("--refine", action="store_true",
                    help="finer moduli-fraction pass over the width's table (classes 0-2)")
    ap.add_argument("--pairs", type=int, default=4096)
    ap.add_argument("--seed", type=int, default=3)
    ap.add_argument("--big-pairs", type=int, default=24)
    ap.add_argument("--big-bits", type=int, default=300000)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--out", default=None)
    ap.add_argument("--log", default=None)
    args = ap.parse_args()
    if args.compare_widths:
        compare_widths(args)
        return
    if args.refine:
        refine(args)
        return

    us, vs, _ = wl.mixed_batch(args.pairs, seed=args.seed)
    by = {c: ([], []) for c in range(4)}
    for u, v in zip(us, vs):
        c = class_of(u, v, args.L)
        by[c][0].append(u)
        by[c][1].append(v)
    bu, bv, _ = wl.serve_requests(args.big_pairs, 1.0, seed=args.seed + 1, big_frac=1.0, big_bits=args.big_bits)
    by[3] = (bu, bv)

    dev = mg.Device(0, args.L)
    log = []
    best = {}
    full = mg.pack_pairs(us, vs)
    full_exp = [math.gcd(u, v) for u, v in zip(us, vs)]
    for c in (2, 1, 0, 3):
        cu, cv = by[c]
        if not cu:
            continue
        if c < 3:   # whole batch, other classes at their current setting
            packed, exp = full, full_exp
            cands = [(t, k, s, 0) for t in (256, 512, 1024) for k in (1, 2, 4) for s in SCALES] + \
                    [(512, 8, s, 0) for s in SCALES] + \
                    [(t, k, s, cs) for t in (512, 1024) for k in (2, 4) for s in SCALES[:3] for cs in (2, 4)]
        else:
            packed, exp = mg.pack_pairs(cu, cv), [math.gcd(u, v) for u, v in zip(cu, cv)]
            cands = [(t, 1, 1.0, cs) for t in (512, 1024) for cs in (4, 8, 16)] + \
                    [(t, k, 1.0, cs) for t in (512, 1024) for k in (2, 4) for cs in (4, 8, 16)]
        for t, k, s, cs in cands:
            dev.set_size_class(c, t, k, s)
            dev.set_class_cluster(c, cs)
            try:
                ms = time_config(dev, packed, exp, args.reps)
            except mg.GcdError as e:       # e.g. a launch shape that does not fit
                log.append({"class": c, "threads": t, "k": k, "nq_scale": s, "cluster": cs, "error": str(e)})
                continue
            log.append({"class": c, "pairs": len(cu), "timed_pairs": len(exp), "threads": t, "k": k,
                        "nq_scale": s, "cluster": cs, "ms": ms})
            print(json.dumps(log[-1]), flush=True)
            if c not in best or ms < best[c][0]:
                best[c] = (ms, t, k, s, cs)
        _, t, k, s, cs = best[c]
        dev.set_size_class(c, t, k, s)
        dev.set_class_cluster(c, cs)
    out = args.out or os.path.join(HERE, "tuning", "gb300_L%d.txt" % args.L)
    os.makedirs(os.path.dirname(out), exist_ok=True)
    dev.save_tuning(out)
    if args.log:
        with open(args.log, "w") as f:
            json.dump({"best": {str(c): b for c, b in best.items()}, "runs": log}, f, indent=1)
    print(open(out).read())
    dev.close()


if __name__ == "__main__":
    main()
