#!/usr/bin/env python
"""Time to 1e-12 relative residual on the 64^3 shifted 3-D Laplacian.

Workload: 7-point Dirichlet Laplacian on a 64 x 64 x 64 grid (n = 262,144)
plus a diagonal shift of 1e-3, geometric nested-dissection ordering, four
right-hand sides i.i.d. uniform[-1, 1] (numpy PCG64, seed 0).  Synthetic:
the reference publishes no input for this configuration.

A step is one complete time-to-solution pass of the numeric phase with the
inputs already in HBM: value assembly (inmatrix), LU factorisation, solve
and FP64 iterative refinement until max_j ||b_j - A x_j|| / ||b_j|| <= 1e-12.
The headline `value` is the mixed form (FP32 factor and solves, FP64
residual and correction); the plain FP64 form is timed beside it.  `e2e`
repeats the mixed step through the public API with pinned host buffers,
host<->device copies inside the timed region.  Ordering and symbolic
factorisation are host work done once per pattern and reported apart.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl reference]
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import tempfile
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
for _p in (ROOT, os.path.join(ROOT, "sparspak.jl_gb300")):
    if _p not in sys.path:
        sys.path.insert(0, _p)

import numpy as np  # noqa: E402

METRIC = "time to 1e-12 rel. residual, mixed vs FP64 on 1 GB300; factor GFLOP/s"
TOL = 1e-12


def parse():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=5)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--grid", type=int, default=64)
    ap.add_argument("--nrhs", type=int, default=4)
    ap.add_argument("--sample-grid", type=int, default=48, help="grid of the CPU baseline's bounded sample")
    ap.add_argument("--ordering", default="nd_grid", choices=["nd_grid", "nd_graph"],
                    help="nested dissection: geometric (box grid) or level-structure (general graph)")
    ap.add_argument("--one-step", action="store_true",
                    help="profiling aid: one warm-up step, then exactly one mixed step, no other work")
    ap.add_argument("--precision", default="fp32", choices=["fp32", "fp64", "bf16s"], help="precision of --one-step")
    ap.add_argument("--config", default="laplace3d", choices=["laplace3d", "batched"],
                    help="laplace3d: the headline 64^3 workload; batched: 512 independent SPD systems (solves/s)")
    ap.add_argument("--batch", type=int, default=512, help="systems of the batched workload (512; fewer for profiling)")
    return ap.parse_args()


def peaks():
    path = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(path):
        with open(path) as f:
            d = json.load(f)
        return d, "measured"
    return {"hbm_gbs": 6800.0, "bf16_tflops": 1900.0, "bf16_tflops_sustained": 1700.0}, "fallback"


class Clocks:
    """nvidia-smi sampling (every 200 ms) during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index):
        self.gpu = gpu_index
        self.f = tempfile.NamedTemporaryFile("w+", suffix=".csv", delete=False)
        self.p = None

    def __enter__(self):
        try:
            self.p = subprocess.Popen(["nvidia-smi", f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                                       "-i", str(self.gpu), "-lms", "200"], stdout=self.f, stderr=subprocess.DEVNULL)
        except OSError:
            self.p = None
        return self

    def __exit__(self, *exc):
        if self.p:
            self.p.terminate()
            self.p.wait(timeout=10)

    def summary(self):
        self.f.flush()
        rows = []
        with open(self.f.name) as fh:
            for line in fh:
                parts = [x.strip() for x in line.split(",")]
                if len(parts) >= 9:
                    rows.append(parts)
        os.unlink(self.f.name)
        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        smax = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[i] for r in rows for i in range(4) if r[5 + i].lower() == "active"})
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": reasons, "samples": len(rows)}


def workload(k, nrhs):
    import sparspak as S

    A = S.gallery.laplacian((k, k, k), shift=1e-3)
    b = S.gallery.random_rhs(A.shape[0], nrhs, seed=0)
    return A, np.asfortranarray(b.reshape(A.shape[0], nrhs))


def orderfunction(ordering, k):
    import sparspak as S

    return S.nd_grid(k, k, k) if ordering == "nd_grid" else S.nd_graph()


def symbolic(A, k, ordering="nd_grid"):
    import sparspak as S

    s = S.SparseSolver(A)
    t0 = time.perf_counter()
    S.findorder_(s, orderfunction(ordering, k))
    t1 = time.perf_counter()
    S.symbolicfactor_(s)
    t2 = time.perf_counter()
    return s, {"order_s": t1 - t0, "symbolic_s": t2 - t1}


def lu_flops(b):
    w = np.diff(b.xsuper)
    ln = np.diff(b.xlindx)
    c = np.concatenate([ln[i] - np.arange(w[i]) for i in range(b.nsuper)]).astype(np.float64)
    return float(np.sum((c - 1) + 2.0 * (c - 1) ** 2))


def chol_flops(b):
    """Cholesky flops sum_j 1 + (c_j - 1) + (c_j - 1) c_j over the column counts."""
    w = np.diff(b.xsuper)
    ln = np.diff(b.xlindx)
    c = np.concatenate([ln[i] - np.arange(w[i]) for i in range(b.nsuper)]).astype(np.float64)
    return float(np.sum(1.0 + (c - 1) + (c - 1) * c))


def supernode_flops(b):
    """Per supernode, the LU flop count of its columns: a proxy of the work
    between two supernodes of _lufactor!'s outer loop, used to cut the
    factorisation into slices of similar cost."""
    w = np.diff(b.xsuper)
    ln = np.diff(b.xlindx)
    out = np.empty(b.nsuper)
    for i in range(b.nsuper):
        c = (ln[i] - np.arange(w[i])).astype(np.float64)
        out[i] = np.sum((c - 1) + 2.0 * (c - 1) ** 2)
    return out


def csc1(A):
    return A.indptr.astype(np.int64) + 1, A.indices.astype(np.int64) + 1, np.ascontiguousarray(A.data)


def oracle_run(k, nrhs, slices=1, ordering="nd_grid"):
    """The reference's numeric phase on the host cores, by the oracle alone
    (its own ordering plug-in and structure phase, dense calls through the
    scipy-bundled BLAS/LAPACK): _inmatrix!, _lufactor!, one _triangularsolve!
    per right-hand side, then the FP64 residual as a check (untimed).  The
    timed work is split into `slices` consecutive parts: slice 0 starts with
    _inmatrix!, each slice factors a range of supernodes, the last one also
    runs the solves.  Returns timings (slice_s sums to total_s) and checks."""
    import oracle

    A, b = workload(k, nrhs)
    n = A.shape[0]
    cp, rv, nz = csc1(A)
    t0 = time.perf_counter()
    st = oracle.structure_csc(cp, rv, n, "nd" if ordering == "nd_grid" else "nd_graph", (k, k, k))
    t_struct = time.perf_counter() - t0
    blas = oracle.use_blas(True)
    nslices = max(int(slices), 1)
    cum = np.cumsum(supernode_flops(st))
    bounds = [int(np.searchsorted(cum, cum[-1] * (q + 1) / nslices) + 1) for q in range(nslices)]
    bounds[-1] = st.nsuper
    o = oracle.OracleLU(st)
    marks = [time.perf_counter()]
    o.inmatrix_csc(cp, rv, nz)
    t_in = time.perf_counter() - marks[0]
    for _ in o.factor_slices(bounds):
        marks.append(time.perf_counter())
    t_fac = marks[-1] - marks[0] - t_in
    x = o.solve(b)
    marks[-1] = time.perf_counter()
    t_solve = marks[-1] - marks[0] - t_in - t_fac
    oracle.use_blas(False)
    rr = float(np.max(np.linalg.norm(b - A @ x, axis=0) / np.linalg.norm(b, axis=0)))
    times = list(np.diff(marks))
    return {"n": n, "nnz_A": int(A.nnz), "flops": lu_flops(st), "structure_s": t_struct, "inmatrix_s": t_in,
            "factor_s": t_fac, "solve_s": t_solve, "total_s": float(sum(times)), "slice_s": times, "relres": rr,
            "blas": blas, "iflag": o.iflag}


def cpu_baseline(args, F_full):
    """The oracle (BLAS mode) on the complete numeric phase of the --sample-grid^3
    instance of the same workload, scaled to the full grid by the LU flop ratio."""
    r = oracle_run(args.sample_grid, args.nrhs, ordering=args.ordering)
    rate = r["flops"] / r["factor_s"]
    est_ms = r["total_s"] * F_full / r["flops"] * 1e3
    return {"value": est_ms, "unit": "ms", "cores": int(r["blas"]["threads"]), "kind": "port",
            "sample": (f"oracle (C restatement of the reference's structure phase, _inmatrix!, _lufactor!, "
                       f"_lulsolve!/_luusolve!; dense calls through {r['blas']['library']}, "
                       f"{r['blas']['threads']} threads) on the complete {args.sample_grid}^3 instance of the same "
                       f"workload ({args.nrhs} right-hand sides): {r['total_s']:.2f} s, factor at "
                       f"{rate / 1e9:.2f} GFLOP/s, rel. residual {r['relres']:.1e}; value = that time x "
                       f"{args.grid}^3 LU flops / {args.sample_grid}^3 LU flops"),
            "factor_gflops": rate / 1e9, "cpu": cpu_model()}


def cpu_model():
    parts = {"0xd4f": "Arm Neoverse-V2", "0xd40": "Arm Neoverse-V1", "0xd0c": "Arm Neoverse-N1",
             "0xd8e": "Arm Neoverse-N3", "0xd84": "Arm Neoverse-V3"}
    try:
        with open("/proc/cpuinfo") as f:
            txt = f.read()
        for key in ("model name", "CPU part"):
            for line in txt.splitlines():
                if line.lower().startswith(key.lower()):
                    v = line.split(":", 1)[1].strip()
                    return f"{parts.get(v, v)} x{os.cpu_count()}"
    except OSError:
        pass
    import platform

    return f"{platform.machine()} x{os.cpu_count()}"


def dist_setup(args):
    ws = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if ws > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() and args.impl == "ours" else "gloo"
        if backend == "nccl":
            torch.cuda.set_device(local)
        dist.init_process_group(backend)
    return ws, rank, local


ORDERING_NAMES = {"nd_grid": "nested dissection (geometric, box grid)",
                  "nd_graph": "nested dissection (level-structure separators, general graph)"}


def config_of(k, nrhs, n, nnz_a, ordering="nd_grid"):
    """The workload, identical in both arms' lines."""
    return {"workload": f"laplace3d_{k}^3_shift1e-3_nd_{nrhs}rhs", "n": n, "nnz_A": nnz_a, "nrhs": nrhs,
            "ordering": ORDERING_NAMES[ordering], "maxblocksize": 30,
            "l2": "inputs larger than L2 (the 64^3 FP32 factor is 1.2 GB)", "parallelism": "replicas"}


def run_reference(args):
    """--impl reference: the reference's algorithm for the path on the host
    cores - the oracle (the Julia package cannot run here), with its own
    structure phase and its dense calls through the bundled BLAS/LAPACK, on
    the same 64^3 workload.  The K timed steps are K consecutive slices of
    ONE complete numeric phase (inmatrix, factorisation in supernode ranges
    of about equal flops, the solves of every right-hand side), so `value`,
    their sum, is one complete time to solution at full size; warm-up steps
    run the complete numeric phase of the 16^3 instance."""
    ws, rank, _ = dist_setup(args)
    if rank != 0:
        return
    for _ in range(args.warmup):
        oracle_run(16, args.nrhs, ordering=args.ordering)
    r = oracle_run(args.grid, args.nrhs, slices=args.steps, ordering=args.ordering)
    v = r["total_s"] * 1e3
    line = {"metric": METRIC, "value": v, "unit": "ms", "n_gpus": args.gpus, "steps": args.steps,
            "warmup": args.warmup, "ms_per_step": v / args.steps, "higher_is_better": False,
            "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic", "impl": "reference",
            "config": config_of(args.grid, args.nrhs, r["n"], r["nnz_A"], args.ordering),
            "step": (f"step = one of {args.steps} consecutive slices of a single complete {args.grid}^3 numeric "
                     f"phase (slice 0 with _inmatrix!, the last with the {args.nrhs} solves); value = their sum; "
                     f"warm-up steps: the complete 16^3 instance"),
            "phases_s": {"structure_once_per_pattern": r["structure_s"], "inmatrix": r["inmatrix_s"],
                         "factor": r["factor_s"], "solve": r["solve_s"]},
            "factor_gflops": r["flops"] / r["factor_s"] / 1e9, "relres": r["relres"],
            "cpu_baseline": {"value": v, "unit": "ms", "cores": int(r["blas"]["threads"]), "kind": "port",
                             "sample": (f"the complete {args.grid}^3 workload: oracle (C restatement of the "
                                        f"reference's structure and numeric phases), dense calls through "
                                        f"{r['blas']['library']} with {r['blas']['threads']} threads"),
                             "cpu": cpu_model()},
            "e2e": {"value": v, "unit": "ms", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def config1(args, dev, stream, timed):
    """Config 1: the 2-D 5-point Laplacian on a 100 x 100 grid (n = 10,000),
    one right-hand side U[-1,1] (seed 0), minimum-degree ordering (the
    reference's default): LU and Cholesky (SPD form) factorisations in FP64
    and the time to a solution, on the device."""
    import torch

    import sparspak as S
    from sparspak.sparse_solver import _ensure_engine, _matrix_arrays

    A = S.gallery.laplacian((100, 100))
    n = A.shape[0]
    b = S.gallery.random_rhs(n, 1, seed=0)
    s = S.SparseSolver(A)
    S.findorder_(s)
    S.symbolicfactor_(s)
    eng = _ensure_engine(s.slvr)
    colptr, rowval, nzval = _matrix_arrays(A)
    eng.set_pattern(colptr, rowval, s.slvr.order.rperm, s.slvr.order.rinvp, index_base=1)
    eng.set_stream(stream.cuda_stream)
    nz_d = torch.tensor(nzval, device=dev)
    b_d = torch.tensor(b.reshape(1, n), device=dev)
    x_d = torch.zeros_like(b_d)
    out = {"workload": "laplace2d_100x100_mmd_1rhs", "n": n, "lu_flops": lu_flops(s.slvr),
           "cholesky_flops": chol_flops(s.slvr)}
    for form, flops in (("fp64", out["lu_flops"]), ("fp64+spd", out["cholesky_flops"])):
        def fac():
            eng.load_values(nz_d, form)
            eng.factor(form)

        def sol():
            eng.load_values(nz_d, form)
            return eng.factor_refine(b_d, x_d, form, TOL, 5)

        for _ in range(args.warmup):
            sol()
        ms_f, _ = timed(fac, args.steps)
        ms_s, (it, rr) = timed(sol, args.steps)
        out["lu" if form == "fp64" else "cholesky"] = {"factor_ms": ms_f, "factor_gflops": flops / (ms_f * 1e-3) / 1e9,
                                                       "time_to_1e-12_ms": ms_s, "relres": rr, "corrections": it}
    eng.close()
    return out


def run_ours(args):
    import torch

    import sparspak as S
    from sparspak.sparse_solver import _ensure_engine, _matrix_arrays

    ws, rank, local = dist_setup(args)
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    k, nrhs = args.grid, args.nrhs
    A, b = workload(k, nrhs)
    n = A.shape[0]
    s, host_t = symbolic(A, k, args.ordering)
    F = lu_flops(s.slvr)
    FC = chol_flops(s.slvr)
    eng = _ensure_engine(s.slvr)
    colptr, rowval, nzval = _matrix_arrays(A)
    t0 = time.perf_counter()
    eng.set_pattern(colptr, rowval, s.slvr.order.rperm, s.slvr.order.rinvp, index_base=1)
    host_t["pattern_s"] = time.perf_counter() - t0
    stats = eng.stats()
    stream = torch.cuda.Stream(dev)            # a real stream (the legacy default stream has handle 0)
    torch.cuda.set_stream(stream)
    eng.set_stream(stream.cuda_stream)

    nz_d = torch.tensor(nzval, device=dev)
    b_d = torch.tensor(np.ascontiguousarray(b.T), device=dev)       # (nrhs, n): rows are right-hand sides
    x_d = torch.zeros_like(b_d)

    def step(prec):   # value assembly, then factorisation + refined solve in one call
        eng.load_values(nz_d, prec)
        if prec.startswith("bf16s"):   # plain refinement, then GMRES-IR once it stagnates
            it, rr, used = eng.factor_refine(b_d, x_d, prec, TOL, 200, solver="auto")
            return it, rr, used
        return eng.factor_refine(b_d, x_d, prec, TOL, 30)

    def barrier():
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)

    def timed(fn, reps):
        barrier()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = None
        for _ in range(reps):
            out = fn()
        e1.record(stream)
        barrier()
        return e0.elapsed_time(e1) / reps, out

    if args.one_step:
        step(args.precision)
        torch.cuda.synchronize(dev)
        t0 = time.perf_counter()
        it, rr = step(args.precision)[:2]
        torch.cuda.synchronize(dev)
        print(json.dumps({"one_step_ms": (time.perf_counter() - t0) * 1e3, "precision": args.precision,
                          "corrections": it, "relres": rr, "grid": k}))
        return
    for _ in range(args.warmup):
        step("fp32")
    # which kernel class dominates the mixed step (one untimed step, every launch timed)
    eng.profile(S._native.KERNEL_CLASSES)
    eng.profile_reset()
    step("fp32")
    prof = eng.profile_read()
    dom = max(prof, key=lambda c: prof[c]["ms"])
    eng.profile([])
    step("fp32")

    # headline: launch sequences replayed as CUDA graphs, no per-kernel events
    eng.profile_reset()
    with Clocks(local) as clk:
        ms_mixed, (it_mixed, rr_mixed) = timed(lambda: step("fp32"), args.steps)
    clocks = clk.summary()
    launches = sum(v["launches"] for v in eng.profile_read().values())
    x_mixed = x_d.cpu().numpy().T.copy()
    # live roofline: the same steps with CUDA events around every launch of the dominant class
    # (and of the Schur-complement kernel, the factor's main product)
    eng.profile(sorted({dom, "tc_schur"}))
    eng.profile_reset()
    ms_mixed_eager, _ = timed(lambda: step("fp32"), args.steps)
    live = eng.profile_read()
    eng.profile([])

    # the same step as two calls (spk_factor, then spk_refine): what the fused call saves
    ms_two, _ = timed(lambda: (eng.load_values(nz_d, "fp32"), eng.factor("fp32"), eng.refine(b_d, x_d, "fp32", TOL, 30)),
                      args.steps)
    # factor-only timings for GFLOP/s
    eng.load_values(nz_d, "fp32")
    ms_f32, _ = timed(lambda: (eng.load_values(nz_d, "fp32"), eng.factor("fp32")), args.steps)
    # the BF16 form: BF16 tensor-core rank updates, FP64 refinement / GMRES-IR
    for _ in range(args.warmup):
        step("bf16s")
    ms_bf16, (it_bf16, rr_bf16, used_bf16) = timed(lambda: step("bf16s"), args.steps)
    x_bf16 = x_d.cpu().numpy().T.copy()
    ms_fb16, _ = timed(lambda: (eng.load_values(nz_d, "bf16s"), eng.factor("bf16s")), args.steps)
    eng.profile(["tc_schur", "tc_trail"])
    eng.profile_reset()
    timed(lambda: (eng.load_values(nz_d, "bf16s"), eng.factor("bf16s")), 1)
    live_bf16 = eng.profile_read()
    eng.profile([])
    # the SPD (Cholesky) form of the same matrix: FP32 factor + FP64 refinement, and FP64
    for _ in range(args.warmup):
        step("fp32+spd")
    ms_spd, (it_spd, rr_spd) = timed(lambda: step("fp32+spd"), args.steps)
    x_spd = x_d.cpu().numpy().T.copy()
    ms_fspd, _ = timed(lambda: (eng.load_values(nz_d, "fp32+spd"), eng.factor("fp32+spd")), args.steps)
    step("fp64+spd")
    ms_spd64, (it_spd64, rr_spd64) = timed(lambda: step("fp64+spd"), max(1, args.steps // 2))
    ms_fspd64, _ = timed(lambda: (eng.load_values(nz_d, "fp64+spd"), eng.factor("fp64+spd")), max(1, args.steps // 2))
    for _ in range(args.warmup):
        step("fp64")
    ms_fp64, (it_fp64, rr_fp64) = timed(lambda: step("fp64"), args.steps)
    x_fp64 = x_d.cpu().numpy().T.copy()
    ms_f64, _ = timed(lambda: (eng.load_values(nz_d, "fp64"), eng.factor("fp64")), max(1, args.steps // 2))
    ms_asm32, _ = timed(lambda: eng.load_values(nz_d, "fp32"), args.steps)
    ms_asm64, _ = timed(lambda: eng.load_values(nz_d, "fp64"), args.steps)

    cfg1 = config1(args, dev, stream, timed)
    bat = batched(args, dev, stream, timed)

    # e2e through the public API with pinned host buffers
    nz_h = torch.tensor(nzval).pin_memory().numpy()
    b_h = torch.tensor(b).pin_memory().numpy()
    b_h = np.asfortranarray(b_h)
    x_h = np.zeros_like(b_h, order="F")

    def e2e():
        eng.load_values(nz_h, "fp32")
        return eng.factor_refine(b_h, x_h, "fp32", TOL, 30)

    e2e()
    ms_e2e, (it_e2e, rr_e2e) = timed(e2e, args.steps)
    x_ref = x_d.cpu().numpy().T
    rr_check = float(np.max(np.linalg.norm(b - A @ x_ref, axis=0) / np.linalg.norm(b, axis=0)))

    # max over ranks
    if ws > 1:
        t = torch.tensor([ms_mixed, ms_fp64, ms_e2e], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms_mixed, ms_fp64, ms_e2e = t.tolist()
    if rank != 0:
        return

    pk, pk_kind = peaks()
    import ctypes

    p32, p64, pdm = ctypes.c_double(), ctypes.c_double(), ctypes.c_double()
    S._native.gpu().spk_measure_peaks(ctypes.byref(p32), ctypes.byref(p64), ctypes.byref(pdm))
    simt = {"fp32_fma_tflops": p32.value, "fp64_fma_tflops": p64.value, "fp64_dmma_tflops": pdm.value,
            "how": "spk_measure_peaks: one timed launch of 8 CTAs per SM x 256 threads, 8 independent chains each"}

    def fwd_err(x):
        return float(np.max(np.abs(x - x_fp64)) / np.max(np.abs(x_fp64)))

    def traffic_of(cls, alg_per_launch=None):
        """DRAM bytes per launch of the class's FP32 kernels from the committed ncu summaries: the block-LU
        class from sampled 64^3 launches (DRAM / algorithmic bytes of a one-block launch, scaled by the
        blocks a launch processes), the others from the 40^3 capture."""
        p64 = os.path.join(ROOT, "profiles", "dram_traffic_k_block_lu_laplace3d64.md")
        if cls == "getrf" and alg_per_launch and os.path.exists(p64):
            ratio = None
            for line in open(p64):
                if line.startswith("therefore ") and "x the algorithmic bytes" in line:
                    ratio = float(line.split()[1].rstrip("x"))
            if ratio:
                return ratio * alg_per_launch, (
                    f"64^3: ncu dram__bytes_read.sum + dram__bytes_write.sum of sampled one-block k_block_lu "
                    f"launches is {ratio:.2f}x their algorithmic bytes "
                    f"(profiles/dram_traffic_k_block_lu_laplace3d64.md); scaled by the algorithmic bytes per "
                    f"launch of the class (the same ratio taken for its small-front kernels)")
        names = {"getrf": ("k_block_lu<float>", "k_block_lu_small<float>", "k_leaf_factor<float>"),
                 "panel": ("k_block_panel<float",),
                 "trail": ("k_block_trail<float>",), "schur": ("k_schur<float>",),
                 "tc_trail": ("k_tc_update<0>",), "tc_schur": ("k_tc_update<1>",),
                 "fwd": ("k_fwd<float>", "k_front_solve<float, 1,", "k_fwd_l21<float>", "k_solve_leaf<float, 1>"),
                 "bwd": ("k_bwd<float>", "k_bwd_u12<float>", "k_front_solve<float, 0,", "k_solve_leaf<float, 0>")}.get(cls, ())
        path = os.path.join(ROOT, "profiles", "dram_traffic_laplace3d40_mixed_step.md")
        if not names or not os.path.exists(path):
            return None, None
        launches = nbytes = 0.0
        for line in open(path):
            cells = [c.strip() for c in line.strip().strip("|").split("|")]
            if len(cells) == 7 and cells[0].startswith(names):
                try:
                    launches += float(cells[1])
                    nbytes += (float(cells[4]) + float(cells[5])) * 1e6
                except ValueError:
                    pass
        if launches == 0:
            return None, None
        return nbytes / launches, ("ncu dram__bytes_read.sum + dram__bytes_write.sum per launch, mean over one "
                                   "mixed step of the 40^3 case (profiles/dram_traffic_laplace3d40_mixed_step.md); "
                                   "not captured at 64^3")

    def roofline_of(cls, prof_live, kind="float"):
        d = prof_live[cls]
        if cls in ("tc_schur", "tc_trail"):
            achieved = d["flops"] / (d["ms"] * 1e-3) / 1e12
            roof = {"bound": "tensor", "achieved": achieved, "peak": pk["bf16_tflops_sustained"], "unit": "TFLOP/s",
                    "peak_kind": f"{pk_kind} bf16 dense sustained (kernel timed inside a long step); achieved counts "
                                 f"the algorithmic flops of the rank updates (the FP32 form issues three TF32 MMAs "
                                 f"per term, at half the bf16 rate; the BF16 form one bf16 MMA)",
                    "compute": S._native.KERNEL_UNITS.get(cls, "")}
        elif cls in ("schur", "trail", "panel", "getrf"):
            achieved = d["flops"] / (d["ms"] * 1e-3) / 1e12
            roof = {"bound": "fp32_simt", "achieved": achieved, "peak": simt["fp32_fma_tflops"], "unit": "TFLOP/s",
                    "peak_kind": "FP32 FMA rate of the CUDA cores, measured live (spk_measure_peaks); the kernel "
                                 "computes on CUDA cores, not the tensor pipe",
                    "compute": S._native.KERNEL_UNITS.get(cls, "")}
        else:
            achieved = d["bytes"] / (d["ms"] * 1e-3) / 1e9
            roof = {"bound": "hbm", "achieved": achieved, "peak": pk["hbm_gbs"], "unit": "GB/s",
                    "peak_kind": f"{pk_kind} HBM copy bandwidth"}
        alg = (d["flops"] if roof["bound"] == "tensor" else d["bytes"]) / max(d["launches"], 1)
        traffic, tnote = traffic_of(cls, d["bytes"] / max(d["launches"], 1))
        roof.update({"frac": roof["achieved"] / roof["peak"], "traffic": traffic, "traffic_unit": "bytes/launch",
                     "traffic_note": tnote,
                     "kernel": S._native.KERNEL_NAMES[cls] + f" ({kind})", "launches": d["launches"],
                     "ms_per_launch": d["ms"] / max(d["launches"], 1),
                     "algorithmic_per_launch": alg})
        return roof

    roof = roofline_of(dom, live)
    roof_schur = roofline_of("tc_schur", live)
    roof_schur_bf16 = roofline_of("tc_schur", live_bf16, "bf16 operands")
    nnz_full = float(s.slvr.xlnz[-1] - 1 + s.slvr.xunz[-1] - 1)
    cpu = cpu_baseline(args, F) if ws == 1 else None
    h2d = nzval.nbytes + b.nbytes
    d2h = b.nbytes
    line = {
        "metric": METRIC, "value": ms_mixed, "unit": "ms", "n_gpus": ws, "steps": args.steps, "warmup": args.warmup,
        "ms_per_step": ms_mixed, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
        "dtype": "f32 factor/solve + f64 residual/correction", "data": "synthetic",
        "config": config_of(k, nrhs, n, int(A.nnz), args.ordering),
        "structure": {"nnz_LU": int(nnz_full), "lu_flops": F, "fronts": stats["fronts"], "levels": stats["levels"],
                      "factor_gb_fp32": nnz_full * 4 / 1e9},
        "mixed": {"ms": ms_mixed, "ms_eager_profiled": ms_mixed_eager, "corrections": it_mixed, "relres": rr_mixed,
                  "two_calls_ms": ms_two,
                  "call": "spk_factor_refine (factorisation and refined solve in one call, the first solve's lower "
                          "levels beside the last levels of the factorisation); two_calls_ms: spk_factor then "
                          "spk_refine",
                  "relres_host_check": rr_check,
                  "factor_ms": ms_f32, "factor_gflops": F / (ms_f32 * 1e-3) / 1e9, "assembly_ms": ms_asm32},
        "fp64": {"ms": ms_fp64, "corrections": it_fp64, "relres": rr_fp64, "factor_ms": ms_f64,
                 "factor_gflops": F / (ms_f64 * 1e-3) / 1e9, "assembly_ms": ms_asm64,
                 "factor_frac_of_fp64_fma": F / (ms_f64 * 1e-3) / 1e12 / simt["fp64_fma_tflops"],
                 "factor_frac_of_fp64_dmma": F / (ms_f64 * 1e-3) / 1e12 / simt["fp64_dmma_tflops"]},
        "bf16s": {"ms": ms_bf16, "preconditioned_solves": it_bf16, "solver": used_bf16, "relres": rr_bf16,
                  "factor_ms": ms_fb16, "factor_gflops": F / (ms_fb16 * 1e-3) / 1e9},
        "spd": {"ms": ms_spd, "corrections": it_spd, "relres": rr_spd, "factor_ms": ms_fspd,
                "factor_gflops": FC / (ms_fspd * 1e-3) / 1e9, "fp64_ms": ms_spd64, "fp64_factor_ms": ms_fspd64,
                "fp64_factor_gflops": FC / (ms_fspd64 * 1e-3) / 1e9, "cholesky_flops": FC,
                "form": "SPK_SPD: no interchanges, lower-only (SYRK-like) rank updates, FP32 factor + FP64 "
                        "refinement; GFLOP/s count the Cholesky flops"},
        "forward_error_vs_fp64": {"mixed": fwd_err(x_mixed), "bf16s": fwd_err(x_bf16), "spd": fwd_err(x_spd),
                                  "note": "max-norm, against the FP64 GPU solution of the same step (which the "
                                          "parity tests hold within 1e-10 of the oracle's)"},
        "config1_grid2d_100": cfg1,
        "batched": bat,
        "speedup_mixed_vs_fp64": ms_fp64 / ms_mixed,
        "speedup_bf16s_vs_fp64": ms_fp64 / ms_bf16,
        "measured_peaks": simt,
        "host_once_per_pattern": host_t,
        "profile_mixed_step": {c: {"ms": round(v["ms"], 4), "launches": v["launches"],
                                   "gflops": round(v["flops"] / max(v["ms"], 1e-9) / 1e6, 1),
                                   "gbs": round(v["bytes"] / max(v["ms"], 1e-9) / 1e6, 1)} for c, v in prof.items()},
        "roofline": roof,
        "roofline_schur": roof_schur,
        "roofline_schur_bf16": roof_schur_bf16,
        "cpu_baseline": cpu,
        "e2e": {"value": ms_e2e, "unit": "ms", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h),
                "corrections": it_e2e, "relres": rr_e2e},
        "gpu_launches": int(launches),
        "clocks": clocks,
    }
    print(json.dumps(line))


def batched(args, dev, stream, timed):
    """512 independent SPD systems (9-point weighted Laplacians of s x s grids,
    s ~ U{20..120}, lognormal conductivities, seed 0), one right-hand side each,
    factored and solved together as one block-diagonal system: a step is value
    assembly + FP32 factorisation + solve + FP64 refinement to 1e-12 of every
    system.  The bottom subtrees of all systems go through the persistent leaf
    queue; the options come from spk_autotune (untimed, before the warm-up).
    Metric: systems solved per second."""
    import torch

    import sparspak as S
    from sparspak.sparse_solver import _ensure_engine, _matrix_arrays

    t0 = time.perf_counter()
    nb = args.batch
    A, sizes = S.gallery.batched_diffusion(nb, 20, 120, seed=0)
    n = A.shape[0]
    b = S.gallery.random_rhs(n, 1, seed=3)
    s = S.SparseSolver(A, precision="fp32")
    S.findorder_(s, S.nd_grid_batched(sizes))
    S.symbolicfactor_(s)
    host_s = time.perf_counter() - t0
    eng = _ensure_engine(s.slvr)
    colptr, rowval, nzval = _matrix_arrays(A)
    eng.set_pattern(colptr, rowval, s.slvr.order.rperm, s.slvr.order.rinvp, index_base=1)
    eng.set_stream(stream.cuda_stream)
    nz_d = torch.tensor(nzval, device=dev)
    b_d = torch.tensor(b.reshape(1, n), device=dev)
    x_d = torch.zeros_like(b_d)

    def fac():
        eng.load_values(nz_d, "fp32")
        eng.factor("fp32")

    def step():
        eng.load_values(nz_d, "fp32")
        return eng.factor_refine(b_d, x_d, "fp32", TOL, 30)

    # factor time with the leaf queue off and on (default thresholds), then the tuner's choice
    fac()
    per_queue = {}
    for q in (0, 1):
        eng.set_option("leaf_queue", q)
        fac()
        per_queue[q], _ = timed(fac, max(3, args.steps // 2))
    eng.load_values(nz_d, "fp32")
    opts, tuned_ms = eng.autotune("fp32", reps=3)
    for _ in range(args.warmup):
        step()
    eng.profile_reset()
    ms, (it, rr) = timed(step, args.steps)
    launches = sum(v["launches"] for v in eng.profile_read().values()) / args.steps
    ms_f, _ = timed(fac, args.steps)
    x = x_d.cpu().numpy().reshape(n)
    r = b.reshape(n) - A @ x
    worst, off = 0.0, 0
    for sz in sizes:
        sl = slice(off, off + sz * sz)
        worst = max(worst, float(np.linalg.norm(r[sl]) / np.linalg.norm(b.reshape(n)[sl])))
        off += sz * sz
    eng.close()
    return {"metric": f"solves/s, {nb} SPD systems (FP32 factor + FP64 refinement to 1e-12)",
            "value": nb / (ms * 1e-3), "unit": "systems/s", "ms_per_step": ms, "factor_ms": ms_f,
            "factor_ms_leaf_queue_off": per_queue[0], "factor_ms_leaf_queue_on": per_queue[1],
            "autotune": {"options": opts, "best_factor_ms": tuned_ms,
                         "how": "spk_autotune: median of 3 timed factorisations per option set (leaf queue off/on, "
                                "then 7 tensor-core threshold pairs)"},
            "gpu_launches_per_step": launches, "corrections": it, "relres": rr, "worst_system_relres": worst,
            "workload": f"batched_{nb}_spd_9pt_s20-120_lognormal", "n": n, "nnz_A": int(A.nnz),
            "nnz_LU": int(s.slvr.xlnz[-1] - 1 + s.slvr.xunz[-1] - 1), "ordering": "nested dissection per system",
            "host_order_symbolic_s": host_s}


def run_batched(args):
    """The batched workload alone, as its own line (--config batched)."""
    import torch

    ws, rank, local = dist_setup(args)
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.Stream(dev)
    torch.cuda.set_stream(stream)

    def timed(fn, reps):
        if ws > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize(dev)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        out = None
        for _ in range(reps):
            out = fn()
        e1.record(stream)
        torch.cuda.synchronize(dev)
        return e0.elapsed_time(e1) / reps, out

    out = batched(args, dev, stream, timed)
    ms = out["ms_per_step"]
    if ws > 1:
        t = torch.tensor([ms], device=dev, dtype=torch.float64)
        torch.distributed.all_reduce(t, op=torch.distributed.ReduceOp.MAX)
        ms = t.item()
    if rank != 0:
        return
    print(json.dumps({
        "metric": out["metric"], "value": args.batch * ws / (ms * 1e-3), "unit": "systems/s", "n_gpus": ws,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32 factor/solve + f64 residual/correction", "data": "synthetic",
        "config": {"workload": out["workload"], "n": out["n"], "nnz_A": out["nnz_A"], "nnz_LU": out["nnz_LU"],
                   "ordering": out["ordering"], "parallelism": "replicas"},
        "batched": out}))


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.config == "batched":
        run_batched(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
