"""Schedule tuner for the batched small-system solver.

Measures, on the device, on the batched workload (libmat_gb300.batched_data):
  * the one-launch schedule (every queue drained by one persistent
    cooperative kernel) with each cap on its resident CTAs per SM;
  * the launch-per-queue schedule, every candidate of each (size bucket,
    kind) queue -- the algorithm (register Gauss-Jordan, or the blocked LU
    for buckets 64..128) and a cap on the resident CTAs per SM.  Each queue
    runs as its own launch, one after another, so a queue's time does not
    depend on the other queues' choices and every queue's candidates are
    swept at once, configuration by configuration;
  * for the mixed-precision mode, each queue of orders 33..128 on the
    tensor-core kernel against its best FP32 candidate ("mixed_tc" entries:
    1 where the tensor-core kernel was faster);
and writes the faster schedule (with the fastest candidate per queue) to
libmat_gb300/batched_tune.json, which the library reads at its first batched
call (compiled-in defaults otherwise).

Usage: python -m libmat_gb300.tune_batched [--count N] [--reps R] [--out F]
(needs a GPU; prints the table it writes).
"""
import argparse
import ctypes as C
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
if os.path.dirname(HERE) not in sys.path:
    sys.path.insert(0, os.path.dirname(HERE))

BUCKETS = (16, 32, 64, 96, 128)
CTAS = (0, 1, 2, 3, 4, 6)


def candidates(nb):
    out = [(0, c) for c in CTAS]
    if nb >= 64:
        out += [(1, c) for c in CTAS]
    return out


def kernel_key(name):
    """(nb, kind) of a batched kernel's timing name, or None."""
    parts = name.split("_")
    if not name.startswith("batched_") or not parts[-1].isdigit():
        return None
    return int(parts[-1]), 1 if "spd" in parts else 0


def timings(L, run, reps):
    L.c.matgb_ktime_enable(1)
    for _ in range(reps):
        run()
    L.sync()
    res, i = {}, 0
    name = (C.c_char * 64)()
    while True:
        cnt, ms, fl, by = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
        if L.c.matgb_ktime_get(i, name, 64, C.byref(cnt), C.byref(ms),
                               C.byref(fl), C.byref(by)) != 0:
            break
        key = kernel_key(name.value.decode())
        if key:
            res[key] = ms.value / reps  # per pass of the batch
        i += 1
    L.c.matgb_ktime_enable(0)
    return res


def fused_timing(L, run, reps):
    """Milliseconds per pass of the one-launch kernel (None if absent)."""
    L.c.matgb_ktime_enable(1)
    for _ in range(reps):
        run()
    L.sync()
    i, out = 0, None
    name = (C.c_char * 64)()
    while True:
        cnt, ms, fl, by = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
        if L.c.matgb_ktime_get(i, name, 64, C.byref(cnt), C.byref(ms),
                               C.byref(fl), C.byref(by)) != 0:
            break
        if name.value.decode() == "batched_fused":
            out = ms.value / reps
        i += 1
    L.c.matgb_ktime_enable(0)
    return out


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--count", type=int, default=100000)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--out", default=os.path.join(HERE, "batched_tune.json"))
    args = ap.parse_args()
    import libmat_gb300 as mg
    from libmat_gb300 import batched_data
    L = mg.load("f32")
    L.check(L.c.matgb_init(0), "init")
    w = batched_data.make(args.count)
    d = {k: L.dalloc(v.nbytes) for k, v in w.items()}
    dx, st = L.dalloc(w["b"].nbytes), L.dalloc(4 * args.count)
    for k, v in w.items():
        L.h2d(d[k], v)
    L.sync()

    def run():
        L.check(L.c.matgb_solve_batched_dev(args.count, d["n"], d["oA"], d["A"],
                                            d["ov"], d["b"], dx, d["k"], st),
                "batched")

    # one-launch schedule, per CTA cap (graphs off: the per-kernel timer)
    fused_ms = {}
    for ctas in (0, 1, 2):
        L.c.matgb_batched_schedule(1, ctas, 0)
        run()
        t = fused_timing(L, run, args.reps)
        if t is not None:
            fused_ms[ctas] = t
    L.c.matgb_batched_schedule(0, 0, 1)
    run()  # warm-up (and the first call's one-time set-up)
    best = {}
    table = {}
    ncfg = max(len(candidates(nb)) for nb in BUCKETS)
    for ci in range(ncfg):
        chosen = {}
        for nb in BUCKETS:
            cand = candidates(nb)
            algo, ctas = cand[ci % len(cand)]
            for kind in (0, 1):
                L.check(L.c.matgb_batched_tune(nb, kind, algo, ctas), "tune")
                chosen[nb, kind] = (algo, ctas)
        run()
        t = timings(L, run, args.reps)
        for key, ms in t.items():
            table.setdefault(key, {})[chosen[key]] = ms
            if key not in best or ms < best[key][1]:
                best[key] = (chosen[key], ms)
    # the mixed-precision mode: each queue of orders 33..128 on the
    # tensor-core kernel against its best FP32 candidate
    for (nb, kind), ((algo, ctas), _) in best.items():
        L.check(L.c.matgb_batched_tune(nb, kind, algo, ctas), "tune")
    prev = L.c.matgb_batched_mixed(2)
    run()
    tc = timings(L, run, args.reps)
    L.c.matgb_batched_mixed(prev)
    for v in list(d.values()) + [dx, st]:
        L.dfree(v)
    entries = []
    for (nb, kind), ((algo, ctas), ms) in sorted(best.items()):
        entries.append({"prec": "f32", "nb": nb, "kind": kind, "algo": algo,
                        "ctas_per_sm": ctas, "ms": round(ms, 4)})
    for (nb, kind), ms in sorted(tc.items()):
        if nb >= 64 and (nb, kind) in best:
            entries.append({"prec": "f32", "nb": nb, "kind": kind,
                            "mixed_tc": int(ms < best[nb, kind][1]),
                            "tc_ms": round(ms, 4)})
    queues_ms = sum(ms for _, ms in best.values())
    fctas, fms = min(fused_ms.items(), key=lambda kv: kv[1]) if fused_ms else (0, None)
    fused = int(fms is not None and fms <= queues_ms)
    doc = {"what": "batched solver schedule: fused 1 = one persistent launch "
                   "(fused_ctas_per_sm: its CTA cap per SM, 0 = occupancy "
                   "limit), 0 = a launch per (bucket nb, kind) queue with the "
                   "entries' algo (0 register Gauss-Jordan, 1 blocked LU) and "
                   "ctas_per_sm",
           "fused": fused, "fused_ctas_per_sm": fctas,
           "fused_ms": {str(k): round(v, 4) for k, v in fused_ms.items()},
           "queues_ms": round(queues_ms, 4),
           "workload": f"{args.count} systems, orders U{{4..128}}, f32",
           "entries": entries,
           "sweep_ms": {f"{nb}/{kind}": {f"{a}/{c}": round(v, 4)
                                          for (a, c), v in sorted(tv.items())}
                        for (nb, kind), tv in sorted(table.items())}}
    with open(args.out, "w") as f:
        json.dump(doc, f, indent=1)
    print(json.dumps({"fused": fused, "fused_ms": doc["fused_ms"],
                      "queues_ms": doc["queues_ms"], "entries": entries}))


if __name__ == "__main__":
    main()
