"""Benchmark of libmatgb's dense-solve hot path on one GB300.

Headline workload (mixed_lu_ir_16384_f64): mat_solve's LU solve of an
n = 16384 double-precision system A x = b, 1 right-hand side N(0,1), with
A = U diag(sigma) V^T, U and V the Q factors of Householder QR of seeded
Gaussian matrices and sigma geometrically spaced to condition numbers 1e2,
1e4 and 1e6 (one matrix per condition number, all resident in HBM: 2 GiB
each, larger than the 129 MB L2).  The solver factors in FP32 with the
trailing updates on the tensor cores (FP16 operands with power-of-two
block scales, each split into hi + remainder and multiplied as three
products, FP32 accumulation) and
refines in FP64 on the GPU (FGMRES preconditioned by the factors) until the
backward error |b - A x|_inf / (|A|_inf |x|_inf + |b|_inf) <= n * 2^-53.
One step = one complete solve of one of the three systems (the steps cycle
through the condition numbers); work per step is the HPL count of the
reference's PLU formula (tests/bench/compare/bench_plu.cpp:74-75) plus the
solve, 2n^3/3 + 2n^2 FLOP.  Every step's backward error is checked.

Reported beside it: the plain FP64 GPU LU solve of the same system (the
baseline the mixed solver must beat by 3x), the tensor-core rank-K update's
roofline (achieved TFLOP/s over the measured BF16 peak), an end-to-end figure
through mat_solve_ir with pinned host buffers, the reference's CPU algorithm
on one pinned host core (its NEON path restated, f64, at reduced n), and
secondary workloads: the
plain float32 GEMM and PLU solve at 8192, the SPD solve at 16384 with 64
right-hand sides, and 100,000 batched uneven solves.

Data: the matrices are generated on the GPU with PyTorch (QR in float32,
product in float64 -- the orthogonal factors are exact to ~1e-6, so the
condition numbers hold to that relative accuracy); PyTorch is only the
harness here, the solves run in libmatgb.  Torch tensors are row-major, so
the library (column-major) sees A^T, which has the same singular values.

Prints ONE JSON line.  --impl reference times the reference's CPU algorithm
for the solve instead -- its NEON-path mat_solve restated (oracle/
neon_port.c; the reference's own source is not present where this runs) --
single-threaded on one pinned host core, on a bounded sample of the same
workload (one solve of the largest order that fits the arm's time).
"""
import argparse
import ctypes as C
import json
import os
import shutil
import subprocess
import sys
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = ("LU/Chol solve TFLOP/s at bwd err <= n*eps64 (mixed+IR vs plain); "
          "batched solves/s")
KAPPAS = (1e2, 1e4, 1e6)


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            return json.load(f), "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0,
            "bf16_tflops_sustained": 1700.0}, "fallback"


# directory for the bench's side files (the nvidia-smi clock samples);
# --log-dir overrides it
LOG_DIR = [os.environ.get("TMPDIR") or "/tmp"]


def out_path(name):
    os.makedirs(LOG_DIR[0], exist_ok=True)
    return os.path.join(LOG_DIR[0], name)


class Clocks:
    """nvidia-smi sampling during the timed region."""

    def __init__(self, path):
        self.path, self.proc = path, None

    def __enter__(self):
        if shutil.which("nvidia-smi"):
            q = ("index,clocks.sm,clocks.max.sm,power.draw,"
                 "clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
                 "clocks_event_reasons.hw_thermal_slowdown,"
                 "clocks_event_reasons.sw_thermal_slowdown,"
                 "clocks_event_reasons.sw_power_cap")
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(
                ["nvidia-smi", "--query-gpu=" + q, "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
            time.sleep(0.3)
        return self

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            self.proc.wait()
            self.f.close()

    def summary(self, dev=0):
        if not self.proc or not os.path.exists(self.path):
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown",
                 "sw_power_cap"]
        for line in open(self.path):
            f = [x.strip() for x in line.split(",")]
            if len(f) < 9 or f[0] != str(dev):
                continue
            try:
                sm.append(float(f[1]))
                mx = float(f[2])
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None,
                "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


def ktable(L):
    """Per-kernel event timing collected by the library (name, launches, ms,
    algorithmic flop, algorithmic bytes)."""
    res, i = [], 0
    names = (C.c_char * 64)()
    while True:
        cnt, ms, fl, by = C.c_longlong(), C.c_double(), C.c_double(), C.c_double()
        if L.c.matgb_ktime_get(i, names, 64, C.byref(cnt), C.byref(ms),
                               C.byref(fl), C.byref(by)) != 0:
            break
        res.append((names.value.decode(), cnt.value, ms.value, fl.value, by.value))
        i += 1
    return sorted(res, key=lambda r: -r[2])


# ----------------------------------------------------------------- data
def _preload_torch_linalg():
    """torch loads its CUDA linear-algebra library lazily by soname; under a
    profiler's injection that lookup can fail, so load it by path first."""
    import ctypes
    import glob
    import torch
    for f in glob.glob(os.path.join(os.path.dirname(torch.__file__), "lib",
                                    "libtorch_cuda_linalg.so*")):
        try:
            ctypes.CDLL(f, mode=ctypes.RTLD_GLOBAL)
        except OSError:
            pass


def conditioned_set(n, kappas, seed):
    """A_kappa = U diag(sigma_kappa) V^T on the GPU (torch, float64)."""
    import torch
    _preload_torch_linalg()
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    U, _ = torch.linalg.qr(torch.randn(n, n, device="cuda", dtype=torch.float32,
                                       generator=g))
    V, _ = torch.linalg.qr(torch.randn(n, n, device="cuda", dtype=torch.float32,
                                       generator=g))
    U = U.double()
    V = V.double()
    mats = {}
    for k in kappas:
        sig = k ** (-torch.arange(n, device="cuda", dtype=torch.float64) / (n - 1))
        mats[k] = (U * sig) @ V.T
    b = torch.randn(n, device="cuda", dtype=torch.float64, generator=g)
    del U, V
    torch.cuda.synchronize()
    return mats, b


def spd_set(n, lam_maxes, nrhs, seed):
    """A = Q diag(lambda) Q^T, lambda log-uniform in [1, lam_max]."""
    import torch
    _preload_torch_linalg()
    g = torch.Generator(device="cuda")
    g.manual_seed(seed)
    Q, _ = torch.linalg.qr(torch.randn(n, n, device="cuda", dtype=torch.float32,
                                       generator=g))
    Q = Q.double()
    mats = {}
    for lm in lam_maxes:
        u = torch.rand(n, device="cuda", dtype=torch.float64, generator=g)
        lam = torch.exp(u * np.log(lm))
        A = (Q * lam) @ Q.T
        mats[lm] = (A + A.T) * 0.5
    B = torch.randn(nrhs, n, device="cuda", dtype=torch.float64, generator=g)
    del Q
    torch.cuda.synchronize()
    return mats, B  # B row-major nrhs x n == column-major n x nrhs


def bwd_err_T(A, x, b):
    """Backward error of the system the library solved (A^T x = b)."""
    r = (b - A.T @ x).abs().max().item()
    return r / (A.abs().sum(0).max().item() * x.abs().max().item()
                + b.abs().max().item())


# ----------------------------------------------------------------- headline
def run_headline(args, mg):
    import torch
    L = mg.load("f64")
    n = args.n
    flops = 2 * n ** 3 / 3 + 2 * n * n
    tol = n * 2.0 ** -53
    t0 = time.time()
    mats, b = conditioned_set(n, KAPPAS, 1234)
    gen_s = time.time() - t0
    x = torch.zeros(n, device="cuda", dtype=torch.float64)
    opts = L.ir_opts(lp_format=args.lp)
    rep = mg.MatIRReport()
    seq = [KAPPAS[i % len(KAPPAS)] for i in range(args.steps)]

    def solve(k):
        rc = L.c.matgb_gesv_ir_dev(n, mats[k].data_ptr(), n, b.data_ptr(),
                                   x.data_ptr(), C.byref(opts), C.byref(rep))
        L.check(rc, "gesv_ir")
        return rep.as_dict()

    for i in range(args.warmup):
        solve(KAPPAS[i % len(KAPPAS)])
    L.sync()
    l0 = L.c.matgb_launch_count()
    reps = []
    with Clocks(out_path("bench_clocks.csv")) as clk:
        t_wall = time.perf_counter()
        L.check(L.c.matgb_event_record(0), "ev")
        for k in seq:
            reps.append(solve(k))
        L.check(L.c.matgb_event_record(1), "ev")
        L.sync()
        t_wall = time.perf_counter() - t_wall
        ms = L.c.matgb_event_elapsed_ms(0, 1)
    launches = int(L.c.matgb_launch_count() - l0)
    ms_step = ms / len(seq)
    value = flops / (ms_step * 1e-3) / 1e12
    per_kappa = {}
    for k, r in zip(seq, reps):
        d = per_kappa.setdefault("%g" % k, {"steps": 0, "ms": [], "converged": 1,
                                            "bwd_err_max": 0.0})
        d["steps"] += 1
        d["ms"].append(r["ms_factor"] + r["ms_refine"])
        d["converged"] &= r["converged"]
        d["bwd_err_max"] = max(d["bwd_err_max"], r["backward_error"])
        d["lp_format"] = r["lp_format"]
        d["krylov_steps"] = r["krylov_steps"]
        d["refinements"] = r["refinements"]
        d["ms_factor"] = r["ms_factor"]
        d["ms_refine"] = r["ms_refine"]
    for d in per_kappa.values():
        d["ms"] = float(np.mean(d["ms"]))
    # FP64 oracle solutions: the plain FP64 GPU LU solve of each system
    # (matgb_getrf_dev + matgb_getrs_dev, pinned to the reference's double
    # mat_solve by the parity tests); each one timed for the speed-up
    Aw = torch.empty_like(mats[KAPPAS[0]])
    piv = torch.empty(2 * n, device="cuda", dtype=torch.int32)
    small = torch.randn(512, 512, device="cuda", dtype=torch.float64)
    L.check(L.c.matgb_getrf_dev(512, small.data_ptr(), 512, piv.data_ptr(),
                                piv.data_ptr() + 4 * n), "getrf warm")
    del small
    xref, plain_ms = {}, {}
    for k in KAPPAS:
        xp = torch.empty_like(b)
        Aw.copy_(mats[k])
        torch.cuda.synchronize()
        L.sync()
        L.check(L.c.matgb_event_record(2), "ev")
        L.check(L.c.matgb_getrf_dev(n, Aw.data_ptr(), n, piv.data_ptr(),
                                    piv.data_ptr() + 4 * n), "getrf")
        L.check(L.c.matgb_getrs_dev(n, 1, Aw.data_ptr(), n,
                                    piv.data_ptr() + 4 * n, b.data_ptr(), n,
                                    xp.data_ptr(), n), "getrs")
        L.check(L.c.matgb_event_record(3), "ev")
        L.sync()
        plain_ms["%g" % k] = L.c.matgb_event_elapsed_ms(2, 3)
        xref[k] = xp
    del Aw
    # independent check of the last solve of each condition number: backward
    # error, and forward error against the FP64 oracle solution
    for k in KAPPAS:
        if "%g" % k not in per_kappa:
            continue
        r = solve(k)
        L.sync()
        d = per_kappa["%g" % k]
        d["bwd_err_check"] = bwd_err_T(mats[k], x, b)
        d["fwd_err"] = ((x - xref[k]).abs().max() / xref[k].abs().max()).item()
        d["fwd_err_est"] = r["forward_error_est"]
        d["plain_fp64_bwd_err"] = bwd_err_T(mats[k], xref[k], b)
    all_ok = all(d["converged"] == 1 and d["bwd_err_max"] <= tol
                 for d in per_kappa.values())

    # per-kernel timing over one solve per condition number
    L.c.matgb_ktime_enable(1)
    for k in KAPPAS:
        solve(k)
    L.sync()
    kt = ktable(L)
    L.c.matgb_ktime_enable(0)
    rl = roofline_block(kt)

    # end to end through mat_solve_ir with pinned host buffers (kappa = 1e4),
    # measured before the long FP64 leg below
    A = mats[1e4]
    e2e = e2e_mixed(L, mg, A, b, flops, opts, max(3, min(args.steps, 5)))

    # plain FP64 GPU LU + solve (same API family), timed above per system
    ms_plain = plain_ms["%g" % 1e4]
    plain = {"ms": ms_plain, "ms_per_kappa": plain_ms,
             "tflops": flops / (ms_plain * 1e-3) / 1e12,
             "bwd_err": per_kappa.get("%g" % 1e4, {}).get("plain_fp64_bwd_err"),
             "kappa": 1e4,
             "api": "matgb_getrf_dev + matgb_getrs_dev (f64)",
             "speedup_of_mixed": {kk: plain_ms[kk] / d["ms"]
                                  for kk, d in per_kappa.items()}}
    del xref

    for k in list(mats):
        del mats[k]
    torch.cuda.empty_cache()
    return {
        "value": value, "unit": "TFLOP/s", "ms_per_step": ms_step,
        "wall_ms_per_step": t_wall * 1e3 / len(seq),
        "dtype": "f64 (FP32 factors, FP16 tensor-core updates, FP32 accumulate)",
        "gpu_launches": launches,
        "config": {"workload": f"mixed_lu_ir_{n}_f64", "n": n, "nrhs": 1,
                   "kappas": list(KAPPAS),
                   "factor_format": {3: "three-part fp16 split (hi+mid+lo, 6 products, "
                                        "per-row/column scales)",
                                     2: "fp16 split (hi+lo, 3 products)", 1: "bf16",
                                     0: "fp16", -1: "fp32 simt"}[args.lp],
                   "refinement": "FGMRES (FP64) preconditioned by the factors",
                   "A": "U diag(sigma) V^T, U,V from QR of seeded N(0,1)",
                   "target_bwd_err": tol, "gen_s": round(gen_s, 1),
                   "l2": "inputs larger than L2 (2 GiB per A, 3 resident)"},
        "all_converged_to_target": all_ok, "per_kappa": per_kappa,
        "plain_fp64": plain, "roofline": rl, "e2e": e2e,
        "clocks": clk.summary(), "kernels": [
            {"name": r[0], "launches": r[1], "ms": round(r[2], 3)} for r in kt[:12]],
    }


def kernel_roofline(kt, name, traffic_ratio=None, note=None):
    """Roofline of one kernel from the library's per-kernel event timing:
    achieved algorithmic bytes/s against the measured HBM peak and
    algorithmic FLOP/s against the measured BF16 (tensor) peak; the larger
    fraction is the binding one."""
    pk, src = peaks()
    tot = sum(r[2] for r in kt) or 1.0
    rows = [r for r in kt if r[0] == name]
    if not rows:
        return None
    _, cnt, ms, fl, by = rows[0]
    tflops = fl / (ms * 1e-3) / 1e12 if ms > 0 else 0.0
    gbs = by / (ms * 1e-3) / 1e9 if ms > 0 else 0.0
    tpk = pk.get("bf16_tflops_sustained") or pk.get("bf16_tflops")
    hpk = pk["hbm_gbs"]
    hbm = {"achieved": gbs, "peak": hpk, "unit": "GB/s", "frac": gbs / hpk}
    ten = {"achieved": tflops, "peak": tpk, "unit": "TFLOP/s",
           "frac": tflops / tpk if tpk else None}
    bound = "hbm" if hbm["frac"] >= (ten["frac"] or 0) else "tensor"
    head = hbm if bound == "hbm" else ten
    out = {"kernel": name, "bound": bound, "launches": cnt, "share": ms / tot,
           "ms_total": ms, "achieved": head["achieved"], "peak": head["peak"],
           "unit": head["unit"], "frac": head["frac"],
           "traffic": traffic_ratio * by / cnt if (traffic_ratio and cnt) else None,
           "algorithmic_bytes_per_launch": by / cnt if cnt else None,
           "algorithmic_flop_per_launch": fl / cnt if cnt else None,
           "hbm": hbm, "tensor": ten,
           "peak_source": f"{src} peaks: hbm_gbs, bf16_tflops_sustained "
                          "(kernels timed inside a long step)"}
    if note:
        out["note"] = note
    return out


def roofline_block(kt):
    """The dominant kernel (most GPU time in a solve) is the fused block
    factorisation -- the critical path, bound by the latency of one cluster
    exchange per column, far below both roofs; the split tensor-core update
    beside it is HBM-bound."""
    top = kt[0][0] if kt else None
    rl = kernel_roofline(
        kt, top,
        note="latency-bound panel chain: one cluster-wide pivot exchange "
             "(DSMEM + barrier.cluster) per column; algorithmic bytes = the "
             "144-column block read and written once (2*m*144*4), FLOP = m*144^2"
        if top == "lu_block_fused" else None)
    # DRAM bytes / algorithmic bytes of one full-size tensor-core launch
    # measured with ncu (M = 7904, N = 7760, K = 192, split form: 444.8 MB of
    # 502.7 MB, the rest of the C traffic served by L2); the C traffic grows
    # with M*N, so the per-launch traffic is that ratio times the algorithmic
    # bytes
    tc = next((r[0] for r in kt if r[0].startswith("tc_gemm")), None)
    if rl is not None and tc is not None and tc != top:
        rl["tensor_update"] = kernel_roofline(kt, tc, traffic_ratio=444.76 / 502.7)
    return rl


def e2e_mixed(L, mg, A, b, flops, opts, ke):
    import torch
    n = A.shape[0]
    es = 8
    hA = L.c.matgb_host_alloc(n * n * es)
    hb = L.c.matgb_host_alloc(n * es)
    hx = L.c.matgb_host_alloc(n * es)
    torch.cuda.synchronize()
    L.check(L.c.matgb_memcpy_d2h(hA, A.data_ptr(), n * n * es), "d2h")
    L.check(L.c.matgb_memcpy_d2h(hb, b.data_ptr(), n * es), "d2h")
    L.sync()
    MA = mg.MatStruct(n, n, hA)
    MB = mg.MatStruct(n, 1, hb)
    MX = mg.MatStruct(n, 1, hx)
    rep = mg.MatIRReport()
    L.check(L.c.mat_solve_ir(C.byref(MX), C.byref(MA), C.byref(MB),
                             C.byref(opts), C.byref(rep)), "mat_solve_ir")
    # each call timed on its own (host clock: it includes the copies and the
    # synchronisation); the median is reported, every sample beside it
    samples = []
    detail = []
    ok = 1
    for _ in range(ke):
        t0 = time.perf_counter()
        L.check(L.c.mat_solve_ir(C.byref(MX), C.byref(MA), C.byref(MB),
                                 C.byref(opts), C.byref(rep)), "mat_solve_ir")
        samples.append((time.perf_counter() - t0) * 1e3)
        ok = ok and rep.converged
        detail.append({"ms_factor": round(rep.ms_factor, 2), "ms_refine": round(rep.ms_refine, 2),
                       "krylov_steps": rep.krylov_steps, "lp_format": rep.lp_format})
    ms = float(np.median(samples))
    for p in (hA, hb, hx):
        L.c.matgb_host_free(p)
    return {"value": flops / (ms * 1e-3) / 1e12, "unit": "TFLOP/s",
            "h2d_bytes_per_step": n * n * es + n * es, "d2h_bytes_per_step": n * es,
            "ms_per_step": ms, "ms_samples": [round(v, 2) for v in samples],
            "samples_detail": detail,
            "converged": int(ok),
            "api": "mat_solve_ir (host Mat/Vec, pinned), kappa = 1e4"}


# ----------------------------------------------------------------- secondary
def c2_golden():
    """The reference's outputs on the 8192 plain config (tests/golden), or
    None when the fixture is absent."""
    p = os.path.join(ROOT, "tests", "golden", "c2_8192.npz")
    if not os.path.exists(p):
        return None
    with np.load(p) as z:
        return {k: z[k] for k in z.files}


def run_plain_f32(mg, steps=3, warmup=3):
    """Plain float32 PLU + 16-RHS solve at 8192 and the 8192^3 GEMM.  The
    PLU inputs are the 8192 plain config's (A ~ N(0,1) seed 1002, B seed
    2002, generated on the host and copied in), so the permutation and the
    forward error are checked against the reference's own outputs."""
    from libmat_gb300 import rng
    L = mg.load("f32")
    c = L.c
    n, nrhs, es = 8192, 16, 4
    nA = n * n * es
    g = c2_golden()
    Ah = rng.normal(1002, (n, n), np.float32)
    Bh = rng.normal(2002, (n, nrhs), np.float32)
    dA0 = L.dalloc(nA)
    dAs = [L.dalloc(nA) for _ in range(steps)]
    dB = L.dalloc(n * nrhs * es)
    dX = L.dalloc(n * nrhs * es)
    dpiv = L.dalloc(2 * n * 4)
    L.h2d(dA0, Ah)
    L.h2d(dB, Bh)
    L.sync()

    def step(dA):
        L.check(c.matgb_getrf_dev(n, dA, n, dpiv, dpiv + n * 4), "getrf")
        L.check(c.matgb_getrs_dev(n, nrhs, dA, n, dpiv + n * 4, dB, n, dX, n),
                "getrs")

    for _ in range(warmup):
        L.check(c.matgb_memcpy_d2d(dAs[0], dA0, nA), "d2d")
        step(dAs[0])
    for d in dAs:
        L.check(c.matgb_memcpy_d2d(d, dA0, nA), "d2d")
    L.sync()
    L.check(c.matgb_event_record(0), "ev")
    for d in dAs:
        step(d)
    L.check(c.matgb_event_record(1), "ev")
    L.sync()
    ms = c.matgb_event_elapsed_ms(0, 1) / steps
    flops = 2 * n ** 3 / 3 + nrhs * 2 * n * n
    A = np.empty((n, n), np.float32, order="F")
    B = np.empty((n, nrhs), np.float32, order="F")
    X = np.empty((n, nrhs), np.float32, order="F")
    L.d2h(A, dA0)
    L.d2h(B, dB)
    L.d2h(X, dX)
    A64 = A.astype(np.float64)
    R = B - A64 @ X
    eta = float((np.abs(R).max(0) / (np.abs(A64).sum(1).max() * np.abs(X).max(0)
                                     + np.abs(B).max(0))).max())
    piv = np.empty(2 * n, np.int32)
    L.d2h(piv, dpiv)
    parity = {"golden": g is not None}
    if g is not None:
        xt = g["x_f64"]
        fe = np.abs(X.astype(np.float64) - xt).max(0) / np.abs(xt).max(0)
        fe_ref = np.abs(g["x_f32"].astype(np.float64) - xt).max(0) / np.abs(xt).max(0)
        parity.update({
            "perm_equals_reference": bool(np.array_equal(piv[n:], g["p_f32"])),
            "swaps": int(np.sum(piv[:n] != np.arange(n))),
            "swaps_reference": int(g["s_f32"]),
            "fwd_err": float(fe.max()),
            "fwd_err_reference_f32": float(fe_ref.max()),
            "fwd_err_oracle": "reference double mat_solve of the same system",
            "kappa_inf_est": float(g["kappa_inf_est"])})
    # GEMM 8192^3 (C = A A, fresh output each time; inputs larger than L2)
    dC = dAs[0]
    for _ in range(warmup):
        L.check(c.matgb_gemm_dev(b"N", b"N", n, n, n, 1.0, dA0, n, dA0, n, 0.0,
                                 dC, n), "gemm")
    L.sync()
    L.check(c.matgb_event_record(0), "ev")
    for _ in range(steps):
        L.check(c.matgb_gemm_dev(b"N", b"N", n, n, n, 1.0, dA0, n, dA0, n, 0.0,
                                 dC, n), "gemm")
    L.check(c.matgb_event_record(1), "ev")
    L.sync()
    ms_g = c.matgb_event_elapsed_ms(0, 1) / steps
    for d in [dA0, dB, dX, dpiv] + dAs:
        L.dfree(d)
    return {"plu_solve_8192_f32": {"ms": ms, "tflops": flops / (ms * 1e-3) / 1e12,
                                   "nrhs": nrhs, "bwd_err_max": eta, **parity},
            "gemm_8192_f32": {"ms": ms_g, "tflops": 2 * n ** 3 / (ms_g * 1e-3) / 1e12}}


def run_spd(mg, n=16384, nrhs=64):
    """SPD solve with 64 right-hand sides: mixed Cholesky (FP16 split
    tensor-core SYRK updates) + refinement for lambda log-uniform in [1,1e3]
    and [1,1e6], and the plain FP64 Cholesky solve of each system, which is
    also the FP64 oracle of the mixed solutions' forward error."""
    import torch
    L = mg.load("f64")
    mats, B = spd_set(n, (1e3, 1e6), nrhs, 77)
    X = torch.empty_like(B)
    flops = n ** 3 / 3 + 2 * nrhs * 2 * n * n
    out = {}
    info = torch.zeros(4, device="cuda", dtype=torch.int32)
    for lm, lp in ((1e3, 2), (1e6, 2)):
        key = "lam_1e%d" % int(round(np.log10(lm)))
        opts = L.ir_opts(lp_format=lp)
        rep = mg.MatIRReport()
        for rnd in range(2):
            L.sync()
            t0 = time.perf_counter()
            rc = L.c.matgb_posv_ir_dev(n, nrhs, mats[lm].data_ptr(), n,
                                       B.data_ptr(), n, X.data_ptr(), n,
                                       C.byref(opts), C.byref(rep))
            L.sync()
            ms = (time.perf_counter() - t0) * 1e3
        L.check(rc if rc != -1 else 0, "posv_ir")
        r = rep.as_dict()
        # plain FP64 Cholesky + 64-RHS solve of the same system
        A = mats[lm]
        Aw = A.clone()
        Xp = B.clone()
        torch.cuda.synchronize()
        L.sync()
        t0 = time.perf_counter()
        L.check(L.c.matgb_potrf_dev(n, Aw.data_ptr(), n, info.data_ptr()), "potrf")
        L.check(L.c.matgb_potrs_dev(n, nrhs, Aw.data_ptr(), n, Xp.data_ptr(), n,
                                    info.data_ptr()), "potrs")
        L.sync()
        ms_p = (time.perf_counter() - t0) * 1e3
        # B, X are row-major nrhs x n: row j is right-hand side j
        fe = ((X - Xp).abs().amax(1) / Xp.abs().amax(1)).max().item()
        out[key] = {
            "ms": ms, "tflops": flops / (ms * 1e-3) / 1e12, "ret": rc,
            "converged": r["converged"], "bwd_err": r["backward_error"],
            "fwd_err": fe, "fwd_err_est": r["forward_error_est"],
            "lp_format": r["lp_format"], "refinements": r["refinements"],
            "ms_factor": r["ms_factor"], "ms_refine": r["ms_refine"],
            "plain_fp64_ms": ms_p, "speedup_vs_plain": ms_p / ms}
        del Aw, Xp
    out["plain_fp64"] = {"ms": out["lam_1e3"]["plain_fp64_ms"],
                         "tflops": flops / (out["lam_1e3"]["plain_fp64_ms"] * 1e-3) / 1e12,
                         "api": "matgb_potrf_dev + matgb_potrs_dev (f64)"}
    del mats, X, B
    torch.cuda.empty_cache()
    return {"workload": f"spd_ir_{n}_{nrhs}rhs_f64",
            "fwd_err_oracle": "plain FP64 GPU Cholesky solve of the same system",
            **out}


def run_lu_full(mg, steps=3, warmup=3):
    """mat_lu (full pivoting) on the device at n = 512 and 2048 (float) and
    2048 (double), beside the oracle port of the reference's scalar
    elimination on one core at n = 512 (float)."""
    from oracle.loader import Oracle
    from libmat_gb300 import rng
    out = {}
    for prec, n in (("f32", 512), ("f32", 2048), ("f64", 2048)):
        L = mg.load(prec)
        c = L.c
        es = 4 if prec == "f32" else 8
        nA = n * n * es
        dA0, dA, dp = L.dalloc(nA), L.dalloc(nA), L.dalloc(8 * n)
        L.check(c.matgb_fill_normal_dev(dA0, n * n, 3001), "fill")
        for _ in range(warmup):
            L.check(c.matgb_memcpy_d2d(dA, dA0, nA), "d2d")
            L.check(c.matgb_getrf_full_dev(n, dA, n, dp, dp + 4 * n), "getrf_full")
        tot = 0.0
        for _ in range(steps):
            L.check(c.matgb_memcpy_d2d(dA, dA0, nA), "d2d")
            L.sync()
            L.check(c.matgb_event_record(0), "ev")
            L.check(c.matgb_getrf_full_dev(n, dA, n, dp, dp + 4 * n), "getrf_full")
            L.check(c.matgb_event_record(1), "ev")
            L.sync()
            tot += c.matgb_event_elapsed_ms(0, 1)
        for d in (dA0, dA, dp):
            L.dfree(d)
        ms = tot / steps
        # each step reads and writes its trailing block once; the first
        # launch only reads the whole matrix
        byts = es * (n * n + 2 * (n - 1) * n * (2 * n - 1) / 6)
        out[f"{prec}_n{n}"] = {"ms": ms, "us_per_step": ms * 1e3 / n,
                               "launches": n + 1,
                               "algorithmic_GBs": byts / (ms * 1e-3) / 1e9}
    n = 512
    A = rng.normal(3001, (n, n), np.float32)
    O = Oracle("f32", "port")
    reps, t0 = 0, time.perf_counter()
    while reps < 3:
        O.lu(A)
        reps += 1
    out["cpu_port_f32_n512_ms"] = (time.perf_counter() - t0) / reps * 1e3
    out["cpu_cores"] = 1
    return out


def run_qr(mg, steps=3, warmup=2):
    """mat_qr's device form (Householder, blocked WY) on square 4096 and tall
    8192 x 2048 matrices, float and double, R and Q (m x m).  FLOPs: LAPACK's
    counts, 2mn^2 - 2n^3/3 for the factorisation and 4m^2n - 4mn^2 + 4n^3/3
    for the explicit Q."""
    out = {}
    for prec, m, n in (("f32", 4096, 4096), ("f32", 8192, 2048), ("f64", 4096, 4096)):
        L = mg.load(prec)
        c = L.c
        es = 4 if prec == "f32" else 8
        dA0, dR, dQ = L.dalloc(m * n * es), L.dalloc(m * n * es), L.dalloc(m * m * es)
        L.check(c.matgb_fill_normal_dev(dA0, m * n, 4001), "fill")

        def one():
            L.check(c.matgb_memcpy_d2d(dR, dA0, m * n * es), "d2d")
            L.check(c.matgb_qr_dev(m, n, dR, m, dQ, m), "qr")
        for _ in range(warmup):
            one()
        tot = 0.0
        for _ in range(steps):
            L.check(c.matgb_memcpy_d2d(dR, dA0, m * n * es), "d2d")
            L.sync()
            L.check(c.matgb_event_record(0), "ev")
            L.check(c.matgb_qr_dev(m, n, dR, m, dQ, m), "qr")
            L.check(c.matgb_event_record(1), "ev")
            L.sync()
            tot += c.matgb_event_elapsed_ms(0, 1)
        ms = tot / steps
        fl = 2 * m * n * n - 2 * n ** 3 / 3 + 4 * m * m * n - 4 * m * n * n + 4 * n ** 3 / 3
        out[f"{prec}_{m}x{n}"] = {"ms": ms, "tflops": fl / (ms * 1e-3) / 1e12}
        for d in (dA0, dR, dQ):
            L.dfree(d)
    return out


def run_blas_t(mg, steps=5, warmup=3):
    """mat_gemv_t's device form on a 16384 x 16384 f32 matrix (1.07 GB) and
    on a 4M x 64 one (row chunks), and AXPY over 2^28 f32 entries: HBM-bound,
    inputs far larger than L2.  GB/s of algorithmic bytes."""
    L = mg.load("f32")
    c = L.c
    pk, src = peaks()
    peak = float(pk["hbm_gbs"])
    out = {"hbm_peak_source": src}

    def timed(fn):
        for _ in range(warmup):
            fn()
        L.sync()
        L.check(c.matgb_event_record(0), "ev")
        for _ in range(steps):
            fn()
        L.check(c.matgb_event_record(1), "ev")
        L.sync()
        return c.matgb_event_elapsed_ms(0, 1) / steps

    for m, n in ((16384, 16384), (1 << 22, 64)):
        dA, dx, dy = L.dalloc(m * n * 4), L.dalloc(m * 4), L.dalloc(n * 4)
        L.check(c.matgb_fill_normal_dev(dA, m * n, 11), "fill")
        L.check(c.matgb_fill_normal_dev(dx, m, 12), "fill")
        L.check(c.matgb_fill_normal_dev(dy, n, 13), "fill")
        ms = timed(lambda: L.check(c.matgb_gemv_t_dev(m, n, 1.0, dA, m, dx, 0.5,
                                                      dy), "gemv_t"))
        gbs = 4 * (m * n + m + 2 * n) / (ms * 1e-3) / 1e9
        out[f"gemv_t_{m}x{n}"] = {"ms": ms, "GBs": gbs, "hbm_frac": gbs / peak}
        for d in (dA, dx, dy):
            L.dfree(d)
    n = 1 << 28
    dx, dy = L.dalloc(n * 4), L.dalloc(n * 4)
    L.check(c.matgb_fill_normal_dev(dx, n, 14), "fill")
    L.check(c.matgb_fill_normal_dev(dy, n, 15), "fill")
    ms = timed(lambda: L.check(c.matgb_axpy_dev(n, 1e-3, dx, dy), "axpy"))
    gbs = 12 * n / (ms * 1e-3) / 1e9
    out["axpy_2^28"] = {"ms": ms, "GBs": gbs, "hbm_frac": gbs / peak}
    for d in (dx, dy):
        L.dfree(d)
    out["hbm_peak_GBs"] = peak
    return out


def run_batched(mg, count=100000, steps=5, warmup=3):
    """The 100k-system workload in the plain FP32 mode (the reference's
    operations, pivots and rounding per system) and in the mixed-precision
    mode (tensor-core kernels refined to an FP32-level residual) -- with the
    tuned per-queue routing ("mixed") and with every queue of orders 33..128
    on the tensor cores ("mixed_all_tensor_core"); the plain figures at the
    top level."""
    from libmat_gb300 import batched_data
    L = mg.load("f32")
    arrs = batched_data.make(count)
    ns, offA, offv, A, b, kinds = (arrs[k] for k in ("n", "oA", "ov", "A", "b", "k"))
    totA, totv = A.size, b.size
    d = {k: L.dalloc(v.nbytes) for k, v in arrs.items()}
    dx = L.dalloc(b.nbytes)
    st = L.dalloc(4 * count)
    for k, v in arrs.items():
        L.h2d(d[k], v)
    L.sync()
    byt = 4 * (totA + 2 * totv)
    pk, src = peaks()
    # algorithmic FLOPs of the reference's path: PLU 2n^3/3, Cholesky n^3/3,
    # plus the two triangular solves 2n^2 (the kernels' Gauss-Jordan form
    # does more); the mean intensity (~12 FLOP/B) is above the FP32 FFMA
    # ridge, so the FP32 fraction is given beside the HBM one
    nn = ns.astype(np.float64)
    flops = float(np.sum(np.where(kinds == 0, 2 * nn ** 3 / 3, nn ** 3 / 3) + 2 * nn ** 2))
    fp32_peak = pk.get("fp32_tflops") or L.c.matgb_measure_fma_peak(0)
    from oracle.loader import Oracle
    O64 = Oracle("f64", "port")

    def run():
        L.check(L.c.matgb_solve_batched_dev(count, d["n"], d["oA"], d["A"],
                                            d["ov"], d["b"], dx, d["k"], st),
                "batched")

    def measure(mode):
        mixed = mode > 0
        prev = L.c.matgb_batched_mixed(mode)
        try:
            for _ in range(warmup):
                run()
            L.sync()
            L.check(L.c.matgb_event_record(0), "ev")
            for _ in range(steps):
                run()
            L.check(L.c.matgb_event_record(1), "ev")
            L.sync()
            ms = L.c.matgb_event_elapsed_ms(0, 1) / steps
            stats = (C.c_int(), C.c_int(), C.c_int())
            L.check(L.c.matgb_batched_mixed_stats(*(C.byref(v) for v in stats)))
            # per-queue kernel times of one more pass
            L.c.matgb_ktime_enable(1)
            run()
            L.sync()
            kt = ktable(L)
            L.c.matgb_ktime_enable(0)
        finally:
            L.c.matgb_batched_mixed(prev)
        status = np.empty(count, np.int32)
        L.d2h(status, st)
        x = np.empty(totv, np.float32)
        L.d2h(x, dx)
        # a sample of 100 systems: backward error, and forward error against
        # the FP64 oracle (the reference's mat_solve / mat_solve_spd in double)
        rs = np.random.default_rng(7)
        worst, worst_fe = 0.0, 0.0
        for s in rs.integers(0, count, 100):
            n = ns[s]
            M = A[offA[s]:offA[s] + n * n].reshape(n, n, order="F").astype(np.float64)
            xs = x[offv[s]:offv[s] + n].astype(np.float64)
            bs = b[offv[s]:offv[s] + n]
            worst = max(worst, np.abs(M @ xs - bs).max() /
                        (np.abs(M).sum(1).max() * np.abs(xs).max() + np.abs(bs).max()))
            xt = O64.solve(M, bs) if kinds[s] == 0 else O64.solve_spd(M, bs)[0]
            worst_fe = max(worst_fe, np.abs(xs - xt).max() / np.abs(xt).max())
        gbs = byt / (ms * 1e-3) / 1e9
        tfl = flops / (ms * 1e-3) / 1e12
        out = {"ms": ms, "solves_per_s": count / (ms * 1e-3), "hbm_gbs": gbs,
               "hbm_frac": gbs / pk["hbm_gbs"], "tflops": tfl,
               "fp32_frac": tfl / fp32_peak if fp32_peak else None,
               "status_nonzero": int((status != 0).sum()),
               "bwd_err_sample_max": worst, "fwd_err_sample_max": worst_fe,
               "kernels": [{"name": r[0], "ms": round(r[2], 4)} for r in kt]}
        if mixed:
            out.update({"refinement_corrections": stats[0].value,
                        "unconverged": stats[1].value,
                        "form": ("the queues the tuning table routes (compiled-in: "
                                 "general 97..128)" if mode == 1 else
                                 "every queue of orders 33..128") +
                                " on the tensor-core kernels: matrix in TMEM, blocked "
                                "Gauss-Jordan (32-column panels), transforms and "
                                "trailing updates as TF32 hi + remainder tcgen05 "
                                "products (FP32 accumulate), FP32 refinement to "
                                "|r|/(|A||x|+|b|) <= n 2^-24; the other queues on "
                                "the FP32 kernels"})
        return out

    plain = measure(0)
    mixed = measure(1)
    mixed_all = measure(2)
    for v in list(d.values()) + [dx, st]:
        L.dfree(v)
    fused = L.c.matgb_batched_schedule(-1, -1, -1)
    res = {"workload": "batched_100k_uneven_f32",
           "schedule": ("one persistent cooperative launch, replayed as a "
                        "CUDA graph" if fused else "one launch per (bucket, "
                        "kind) queue, replayed as a CUDA graph"),
           "tune_source": L.c.matgb_batched_tune_source().decode(),
           "bytes": byt, "hbm_peak_source": src, "flops": flops,
           "fp32_peak_tflops": fp32_peak,
           "fwd_err_oracle": "reference mat_solve / mat_solve_spd in double "
                             "(oracle port), 100 sampled systems"}
    res.update(plain)
    res["mixed"] = mixed
    res["mixed_all_tensor_core"] = mixed_all
    return res


# ----------------------------------------------------------------- CPU legs
# The reference's own CPU path for the headline's solve (mat_solve in double)
# is timed through oracle/neon_port.c: the reference's NEON-path algorithm
# restated (blocked PLU with its packed 8 x 4 GEMM micro-kernel), which takes
# the NEON micro-kernel on the GPU host's Grace cores.  The reference's own
# source is not present on that host, so its build cannot run there.  One
# pinned core, as the reference is single-threaded.


def _pin_one_core():
    cpus = sorted(os.sched_getaffinity(0))
    core = cpus[-1]
    os.sched_setaffinity(0, {core})
    return core


def _cpu_solver(own=False):
    """The timed CPU solve: the NEON-path restatement of the reference's
    mat_solve (oracle/neon_port.c; the conservative baseline -- the
    reference's own double NEON path does not compile on aarch64, so its own
    double build there is its slower SCALAR path), or with own=True the
    reference's own mat_solve built from its header (the copy in
    oracle/_ref/src travels to the GPU host; -O3, single-threaded).
    Returns (solve, arch, kind, what) or None when own=True and that build
    is absent."""
    from oracle import loader
    if own:
        try:
            if loader.ref_dir() and not loader.available("f64", "time"):
                loader.build()
            if loader.available("f64", "time"):
                o = loader.Oracle("f64", "time")
                return (o.solve, o.arch(), "reference",
                        "the reference's own mat_solve (its mat.h built with -O3, "
                        "single-threaded)")
        except Exception:
            pass
        return None
    N = loader.NeonPort()
    return (N.solve, N.arch(), "port",
            "reference mat_solve algorithm (NEON path: blocked PLU with the packed "
            "8x4 micro-kernel, restated in oracle/neon_port.c)")


def _neon_worker(n_list, budget_s, seed, q, own=False):
    """In a fresh process pinned to one core: time the reference's mat_solve
    at the largest order in n_list that finishes within budget_s, return
    (n, seconds per solve, solves, arch, core, kind, what), or None."""
    core = _pin_one_core()
    from libmat_gb300 import rng
    got = _cpu_solver(own)
    if got is None:
        q.put(None)
        return
    solve, arch, kind, what = got
    # calibrate on the smallest order
    n0 = n_list[0]
    A = rng.normal(seed, (n0, n0), np.float64)
    b = rng.normal(seed + 1, (n0,), np.float64)
    t0 = time.perf_counter()
    solve(A, b)
    t_n0 = time.perf_counter() - t0
    n = n0
    for cand in n_list:
        if t_n0 * (cand / n0) ** 3 * 3 <= budget_s:
            n = cand
    A = rng.normal(seed + 2, (n, n), np.float64)
    b = rng.normal(seed + 3, (n,), np.float64)
    reps, t0 = 0, time.perf_counter()
    while True:
        solve(A, b)
        reps += 1
        el = time.perf_counter() - t0
        if el > budget_s * 0.5 or reps >= 20:
            break
    q.put((n, el / reps, reps, arch, core, kind, what))


def neon_sample(n_list=(1024, 2048, 3072, 4096), budget_s=20.0, seed=1001, own=False):
    import multiprocessing as mp
    ctx = mp.get_context("spawn")
    q = ctx.Queue()
    p = ctx.Process(target=_neon_worker, args=(n_list, budget_s, seed, q, own))
    p.start()
    out = q.get(timeout=budget_s * 10 + 120)
    p.join()
    return out


def own_build_sample():
    """The reference's own double build on this host, timed beside the
    baseline (None where it is absent)."""
    got = neon_sample((512, 1024, 2048), budget_s=10.0, seed=1101, own=True)
    if got is None:
        return None
    n, per, reps, arch, core, _, what = got
    flops = 2 * n ** 3 / 3 + 2 * n * n
    out = {"value": flops / per / 1e12, "unit": "TFLOP/s", "cores": 1,
           "mat_arch": arch,
           "sample": f"{what} in f64 at n={n}, {reps} solves, {per:.2f} s per "
                     f"solve, core {core} pinned"}
    import platform
    if arch != "NEON" and platform.machine() in ("aarch64", "arm64"):
        out["note"] = ("its double NEON path does not compile on aarch64 (gcc 13: "
                       "vfmaq_laneq_f64 lanes 2 and 3 of a two-lane vector, "
                       "mat.h:5439-5440): this is its SCALAR path")
    return out


def cpu_sample():
    """The reference's mat_solve in double on one pinned host core, at the
    largest order that fits a ~20 s budget (the NEON-path restatement), with
    the reference's own build timed beside it.  TFLOP/s."""
    n, per, reps, arch, core, kind, what = neon_sample()
    flops = 2 * n ** 3 / 3 + 2 * n * n
    return {"value": flops / per / 1e12, "unit": "TFLOP/s", "cores": 1,
            "kind": kind,
            "sample": f"{what} in f64 at n={n}, {reps} solves, "
                      f"{per:.2f} s per solve, core {core} pinned",
            "mat_arch": arch, "reference_own_build": own_build_sample()}


def run_reference(args):
    """Reference arm: the reference's CPU algorithm for the headline solve
    (mat_solve in double, its NEON path as restated in oracle/neon_port.c --
    its own double NEON code does not compile on aarch64), single-threaded on
    one pinned host core as the reference runs; each step one solve at the
    largest order whose warm-up + timed steps fit about two minutes.  The
    reference's own double build (its SCALAR path there) is timed beside it."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    core = _pin_one_core()
    from libmat_gb300 import rng
    solve, arch, kind, what = _cpu_solver()
    total = max(1, args.steps + args.warmup)
    n0 = 1024
    A = rng.normal(7, (n0, n0), np.float64)
    b = rng.normal(8, (n0,), np.float64)
    t0 = time.perf_counter()
    solve(A, b)
    t_n0 = time.perf_counter() - t0
    n = n0
    for cand in (1024, 1536, 2048, 3072, 4096, 6144, 8192):
        if t_n0 * (cand / n0) ** 3 * total <= 120.0:
            n = cand
    flops = 2 * n ** 3 / 3 + 2 * n * n
    for i in range(args.warmup):
        solve(rng.normal(100 + i, (n, n), np.float64),
              rng.normal(200 + i, (n,), np.float64))
    mats = [(rng.normal(5000 + i, (n, n), np.float64),
             rng.normal(6000 + i, (n,), np.float64)) for i in range(min(args.steps, 3))]
    t0 = time.perf_counter()
    for i in range(args.steps):
        A, b = mats[i % len(mats)]
        solve(A, b)
    el = time.perf_counter() - t0
    tf = flops * args.steps / el / 1e12
    sample = f"one f64 solve of n={n} per step ({what}), core {core} pinned"
    line = {
        "impl": "reference", "metric": METRIC, "value": tf, "unit": "TFLOP/s",
        "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": el / args.steps * 1e3, "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": {"workload": "mixed_lu_ir_16384_f64", "sample": sample},
        "cpu_baseline": {"value": tf, "unit": "TFLOP/s", "cores": 1,
                         "kind": kind, "sample": sample, "mat_arch": arch,
                         "reference_own_build": own_build_sample()},
        "e2e": {"value": tf, "unit": "TFLOP/s", "h2d_bytes_per_step": 0,
                "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=6)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--n", type=int, default=16384)
    ap.add_argument("--lp", type=int, default=2,
                    help="3 three-part FP16 split (6 products), 2 FP16 split (3 "
                         "products), 0 FP16, 1 BF16, -1 FP32")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-secondary", action="store_true")
    ap.add_argument("--only", choices=["plain_f32", "spd", "batched", "lu_full", "blas_t",
                                       "qr"],
                    help="run one secondary workload alone and print its JSON "
                         "(small cases for profiling)")
    ap.add_argument("--count", type=int, default=100000,
                    help="systems in the batched workload")
    ap.add_argument("--log-dir", default=None,
                    help="where side files (clock samples) are written "
                         "(default $TMPDIR or /tmp)")
    args = ap.parse_args()
    if args.log_dir:
        LOG_DIR[0] = args.log_dir
    if args.impl == "reference":
        return run_reference(args)
    if args.only:
        import libmat_gb300 as mg
        for p in ("f32", "f64"):
            if mg.load(p).c.matgb_init(0) != 0:
                raise SystemExit("matgb_init failed")
        if args.only == "plain_f32":
            out = run_plain_f32(mg, steps=args.steps, warmup=args.warmup)
        elif args.only == "spd":
            out = run_spd(mg, n=args.n)
        elif args.only == "blas_t":
            out = run_blas_t(mg, steps=args.steps, warmup=args.warmup)
        elif args.only == "lu_full":
            out = run_lu_full(mg, steps=args.steps, warmup=args.warmup)
        elif args.only == "qr":
            out = run_qr(mg, steps=args.steps, warmup=args.warmup)
        else:
            out = run_batched(mg, count=args.count, steps=args.steps,
                              warmup=args.warmup)
        print(json.dumps(out), flush=True)
        return
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    import torch
    torch.cuda.set_device(local)
    import libmat_gb300 as mg
    for p in ("f32", "f64"):
        if mg.load(p).c.matgb_init(local) != 0:
            raise SystemExit("matgb_init failed: %s" % mg.load(p).c.matgb_last_error())
    res = run_headline(args, mg)
    if world > 1:
        # replicas only: every rank solves the same independent systems; the
        # whole-job value is the sum over ranks timed by the slowest rank
        import torch.distributed as dist
        dist.init_process_group("gloo")
        t = [None] * world
        dist.all_gather_object(t, res["ms_per_step"])
        dist.destroy_process_group()
        res["ms_per_step"] = max(t)
        res["value"] = (2 * args.n ** 3 / 3 + 2 * args.n ** 2) * world / \
            (res["ms_per_step"] * 1e-3) / 1e12
    if rank != 0:
        return
    secondary = None
    if not args.no_secondary:
        secondary = {"plain_f32": run_plain_f32(mg), "spd": run_spd(mg),
                     "batched": run_batched(mg), "lu_full": run_lu_full(mg),
                     "qr": run_qr(mg), "blas_t": run_blas_t(mg)}
    cpu = None
    if not args.no_cpu:
        cpu = cpu_sample()
    line = {"metric": METRIC, "value": res["value"], "unit": res["unit"],
            "n_gpus": world, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": res["ms_per_step"], "higher_is_better": True,
            "scaling": "weak", "vs_baseline": None, "dtype": res["dtype"],
            "data": "synthetic", "config": res["config"],
            "all_converged_to_target": res["all_converged_to_target"],
            "per_kappa": res["per_kappa"], "plain_fp64": res["plain_fp64"],
            "roofline": res["roofline"], "cpu_baseline": cpu, "e2e": res["e2e"],
            "gpu_launches": res["gpu_launches"], "clocks": res["clocks"],
            "kernels": res["kernels"], "secondary": secondary,
            "wall_ms_per_step": res["wall_ms_per_step"]}
    print(json.dumps(line), flush=True)


if __name__ == "__main__":
    main()
