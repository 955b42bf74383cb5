#!/usr/bin/env python
"""Benchmark of the GB300 local SpGEMM / SpMSpV path.

Default workload (the headline): C = A*A on an R-MAT of scale 20, edge
factor 16 (a,b,c,d = .57,.19,.19,.05, symmetrized, no self-loops, seeded),
PlusTimes over fp64 with int64 indices, computed in column phases because
nnz(C) ~ 2.4e10 exceeds device memory; each phase's output is written to
HBM and reduced to checksums.  Phases are sized by the learned sizing
network (trained, untimed, on another seed's exact counts); the exact
two-phase path is timed beside it and must produce the same product (nnz,
row checksum, 64-bit content hash).  Metric: Gmults/s (multiplications as
the reference's estimateFLOP counts them, divided by time).  The line also
carries BFS GTEPS on the same graph (64 seeded roots, SelectMin parents) and
the MCL expansion step (n = 2^20, fp32) exact vs learned.

The default run also measures every other configuration in the same line
(``configs``): C1 (R-MAT s14 A*A), C2 (BFS s20, top-down and
direction-optimizing), C3 (MCL expansion n = 2^20), C4 (the 256-problem
uneven batch) and C5 (multi-source BFS s22, 512 roots), each with its own
roofline, CPU baseline, end-to-end figure and a parity check against the
oracle; ``parity`` collects them together with the headline's own check
(the s20 product on a 4096-column sample, bit-exact under both folds).
``--headline-only`` skips them.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
                  [--workload spgemm20|bfs20|spgemm14] [--scale S] [--no-mcl] [--no-cpu]

--impl reference times the CPU implementation of the same path on the host
cores (the oracle's C restatement of the reference's algorithm, OpenMP over
all cores) on a bounded column sample of the same workload.

N > 1 runs independent replicas, one per GPU (the path is not sharded here).
"""
from __future__ import annotations

import argparse
import json
import os
import statistics
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

SEED = 1
BFS_ROOTS = 64
# DRAM bytes of k_numeric_x measured by ncu on a scale-20 column sample
# (profiles/k_numeric_x_s20_cols4096.txt), used to scale roofline.traffic
NUMERIC_DRAM_READ_PER_MULT = 6.23
NUMERIC_DRAM_WRITE_PER_ENTRY = 17.34
# The compiled reference's own hybrid path (heap columns below compression
# ratio 2, hash above, mtSpGEMM.h:310-311) against the restatement timed here,
# same samples and threads (8 x86 cores): s20 A*A(:, 4096 columns) 4.05 s vs
# 3.82 s, s14 A*A 0.487 s vs 0.468 s.
CPU_CALIBRATION = "the compiled reference's hybrid path needs 1.04-1.06x the port's time on the same samples"
# DRAM bytes of the multi-source BFS kernels per scanned edge (expand +
# finalize) as last captured, when each level was a separate graph launch
# (profiles/launches_msbfs22.txt); the traversal is now one graph whose
# level kernels run inside a conditional while node, which ncu does not
# list as launches, so the line reports no traffic of its own.
MSBFS_DRAM_PER_SCANNED_EDGE_LEVEL_REPLAY = 19.5
MS_ROOTS = 512


def log(*a):
    print(*a, file=sys.stderr, flush=True)


# ----------------------------------------------------------------- clocks
class ClockSampler:
    """nvidia-smi clocks / throttle reasons sampled while the timed region runs."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device: int):
        self.device = device
        self.proc = None
        self.lines: list[str] = []

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.thread = threading.Thread(target=self._read, daemon=True)
            self.thread.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.lines:
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for name, flag in zip(names, p[5:9]):
                if flag.lower() == "active":
                    reasons.add(name)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


# ---------------------------------------------------------------- helpers
def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        d = json.load(open(p))
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def bytes_alg(nnzA, n, nnzC, s_i=8, s_v=8):
    """Algorithmic bytes of one SpGEMM A*A: A and B read once, C written once."""
    return 2 * (nnzA * (s_i + s_v) + (n + 1) * s_i) + nnzC * (s_i + s_v) + (n + 1) * s_i


def column_sample(A, frac: float, seed: int = 7):
    """B = A(:, cols) for a seeded random subset of columns (CSC)."""
    from combblas_gb300.generators import CSC

    rng = np.random.default_rng(seed)
    k = max(1, int(A.ncol * frac))
    cols = np.sort(rng.choice(A.ncol, k, replace=False))
    cnt = np.diff(A.colptr)[cols]
    cp = np.concatenate([[0], np.cumsum(cnt)]).astype(np.int64)
    idx = np.concatenate([np.arange(A.colptr[c], A.colptr[c + 1]) for c in cols]) if k else np.zeros(0, np.int64)
    return CSC(A.nrow, k, cp, A.rowidx[idx], None if A.values is None else A.values[idx]), cols


def cpu_spgemm_rate(A, budget_s: float):
    """Oracle (C restatement, all host threads) on a column sample sized for
    ~budget_s seconds: returns (Gmults/s, sample description, threads)."""
    import oracle as O

    frac = 1.0 / 4096
    while True:
        B, cols = column_sample(A, frac)
        t0 = time.perf_counter()
        (_, _, _), (flop, cnt) = O.port_spgemm(A, B, O.SR_PLUSTIMES_F64, want_counts=True)
        dt = time.perf_counter() - t0
        if dt > budget_s / 4 or frac >= 1.0:
            break
        frac = min(1.0, frac * max(2.0, budget_s / 2 / max(dt, 1e-3)))
    flops = int(flop.sum())
    return flops / dt / 1e9, f"A*A(:,{len(cols)} seeded random columns) = {flops:.3e} mults in {dt:.2f}s", \
        O.port_num_threads()


def cpu_bfs_rate(A, roots, budget_s: float):
    import oracle as O

    P = A.with_values(None)
    deg = np.diff(P.colptr)
    edges, secs, used = 0, 0.0, 0
    for r in roots:
        t0 = time.perf_counter()
        par, lev, it = O.port_bfs(P, int(r), with_levels=True)
        secs += time.perf_counter() - t0
        reached = (par >= 0)
        reached[int(r)] = True
        edges += int(deg[reached].sum()) // 2
        used += 1
        if secs > budget_s:
            break
    return edges / secs / 1e9, f"{used} BFS roots", O.port_num_threads()


def cpu_batch_rate(budget_s: float):
    """Oracle restatement over the batch's problems in order until about
    budget_s seconds: Gmults/s."""
    import oracle as O
    from combblas_gb300 import generators as G

    rm, gk = G.batch_c4(256, seed=4)
    pairs = [(A, A) for A in rm] + [(A, Rt) for A, R, Rt in gk]
    order = np.random.default_rng(SEED).permutation(len(pairs))
    flops, secs, used = 0, 0.0, 0
    for p in order:
        A, B = pairs[p]
        t0 = time.perf_counter()
        (_, _, _), (fl, _) = O.port_spgemm(A, B, O.SR_PLUSTIMES_F64, want_counts=True)
        secs += time.perf_counter() - t0
        flops += int(fl.sum())
        used += 1
        if secs > budget_s:
            break
    return flops / secs / 1e9, f"{used} of the 256 first-stage products (seeded random order)", O.port_num_threads()


def dist_setup(args):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch.distributed as dist

        backend = "nccl" if args.impl == "ours" else "gloo"
        dist.init_process_group(backend)
    return world, rank, local


def max_over_ranks(x: float, world: int, device=None) -> float:
    if world == 1:
        return x
    import torch
    import torch.distributed as dist

    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def make_graph(workload, scale_override=0):
    from combblas_gb300 import generators as G

    scale, ef = {"spgemm14": (14, 8), "msbfs22": (22, 16)}.get(workload, (20, 16))
    if scale_override:
        scale = scale_override
    t0 = time.perf_counter()
    A = G.rmat(scale, ef, seed=SEED)
    log(f"generated R-MAT scale {scale} ef {ef}: n={A.ncol} nnz={A.nnz} in {time.perf_counter() - t0:.1f}s")
    return A, scale, ef


def bfs_roots(A, k=BFS_ROOTS):
    deg = np.diff(A.colptr)
    rng = np.random.default_rng(SEED + 100)
    return rng.choice(np.nonzero(deg)[0], k, replace=False)


# -------------------------------------------------------------- reference
def run_reference(args, world, rank):
    if rank != 0:
        return
    import oracle as O

    O.build(quiet=True) if not os.path.exists(O._PORT_SO) else None
    A, scale, ef = make_graph(args.workload, args.scale) if args.workload != "batch256" else (None, 0, 0)
    budget = 20.0
    steps = []
    desc, threads = "", 1
    if args.workload == "batch256":
        for s in range(args.warmup + args.steps):
            v, desc, threads = cpu_batch_rate(budget / 4)
            if s >= args.warmup:
                steps.append(v)
        metric, unit = metric_name(args.workload, scale, ef), "Gmults/s"
    elif args.workload in ("bfs20", "msbfs22"):
        roots = bfs_roots(A)
        for s in range(args.warmup + args.steps):
            v, desc, threads = cpu_bfs_rate(A, roots[s % len(roots):], budget / 4)
            if s >= args.warmup:
                steps.append(v)
        metric, unit = metric_name(args.workload, scale, ef), "GTEPS"
    else:
        for s in range(args.warmup + args.steps):
            v, desc, threads = cpu_spgemm_rate(A, budget / 2)
            if s >= args.warmup:
                steps.append(v)
        metric, unit = metric_name(args.workload, scale, ef), "Gmults/s"
    val = float(np.median(steps))
    line = {
        "impl": "reference", "metric": metric, "value": val, "unit": unit, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.workload.startswith("spgemm") or args.workload == "batch256" else "int64",
        "data": "synthetic (seeded R-MAT)",
        "config": workload_config(args, scale, ef, world),
        "cpu_baseline": {"value": val, "unit": unit, "cores": threads, "kind": "port",
                         "sample": desc + " per step; the reference's CPU algorithm as restated in oracle/oracle.c "
                                          "(the compiled reference needs sources that the GPU hosts do not carry)",
                         **({"calibration": CPU_CALIBRATION} if args.workload.startswith("spgemm") else {})},
        "e2e": {"value": val, "unit": unit, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args, scale, ef, world):
    """The `config` object of both arms' JSON lines (the same workload)."""
    return {"workload": args.workload, "scale": scale, "edge_factor": ef, "seed": SEED,
            "rmat_abcd": [0.57, 0.19, 0.19, 0.05], "index": "int64",
            "phase_budget_nnz": args.phase_nnz, "l2": "inputs and outputs larger than L2 (129 MB)",
            "parallelism": f"replicas x{world}", **({"b_columns": args.bcols} if args.bcols else {})}


def metric_name(workload, scale, ef):
    if workload == "batch256":
        return "batched SpGEMM Gmults/s (256 uneven problems: R-MAT A*A 2^10..2^18, Galerkin R*A*R^T)"
    if workload == "msbfs22":
        return f"multi-source BFS GTEPS (R-MAT s{scale} ef{ef}, {MS_ROOTS} roots, Select2ndMin SpGEMM loop)"
    if workload == "bfs20":
        return f"BFS GTEPS (R-MAT s{scale} ef{ef}, 64 roots, SelectMin parents)"
    return f"SpGEMM Gmults/s (R-MAT s{scale} ef{ef} A*A, PlusTimes fp64, exact output)"


def train_sizing_model(ctx, scale, ef, Ad_like=None):
    """Sizing network trained (untimed) on the exact column counts of
    another seed's matrix of the same statistics class."""
    from combblas_gb300 import generators as G
    from combblas_gb300 import local as LC
    from combblas_gb300 import sizing as SZ

    t0 = time.perf_counter()
    At = G.rmat(scale, ef, seed=SEED + 1)
    Atd = LC.DeviceMatrix.from_host(At)
    feat, flop, nnz = SZ.features(Atd, Atd, ctx=ctx)
    m = SZ.SizingModel(ctx)
    info = m.fit(feat, nnz, steps=300)
    m.use()
    info["train_seconds"] = time.perf_counter() - t0
    info["trained_on"] = f"R-MAT s{scale} ef{ef} seed {SEED + 1} (exact symbolic counts, {info['samples']} columns)"
    del Atd
    return m, info


def bench_spgemm(args, world, A, Ad, ctx, stream, scale, ef, hbm, peak_kind):
    """Headline: A*A in column phases with learned phase sizing; the exact
    two-phase path is timed beside it and must give the same product
    (nnz, row checksum and 64-bit content hash)."""
    import torch
    from combblas_gb300 import _lib
    from combblas_gb300 import local as LC

    budget = args.phase_nnz
    model, info = train_sizing_model(ctx, scale, ef)

    Bh, Bd = A, Ad
    if args.bcols:  # profiling case: B = A(:, bcols seeded random columns), full row range
        Bh = column_sample(A, args.bcols / A.ncol)[0]
        Bd = LC.DeviceMatrix.from_host(Bh)

    def step(sizing):
        return LC.spgemm_phased(Ad, Bd, max_phase_nnz=budget, ctx=ctx, sizing=sizing)

    def timed(sizing, steps, clocks=None):
        torch.cuda.synchronize()
        barrier(world)
        if clocks:
            clocks.start()
        l0 = _lib.lib().gbc_launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        agg = {"sizing": 0.0, "numeric": 0.0, "rerun": 0.0}
        torch.cuda.nvtx.range_push(f"timed_{sizing}")  # lets ncu --nvtx-include select the timed steps
        e0.record(stream)
        for _ in range(steps):
            st = step(sizing)
            agg["sizing"] += st.ms_sizing
            agg["numeric"] += st.ms_numeric
            agg["rerun"] += st.ms_rerun
        e1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        ms = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
        launches = _lib.lib().gbc_launch_count() - l0
        ck = clocks.stop() if clocks else None
        return st, ms, launches, {k: v / steps for k, v in agg.items()}, ck

    for _ in range(args.warmup):
        step("learned")
    step("exact")
    st, ms, launches, agg, ck = timed("learned", args.steps, ClockSampler(int(torch.cuda.current_device())))
    st_x, ms_x, _, agg_x, _ = timed("exact", args.steps)
    same = (st.nnz, st.row_checksum, st.content_hash) == (st_x.nnz, st_x.row_checksum, st_x.content_hash)
    if not same:
        raise SystemExit("learned and exact phased products differ")
    flops = st.flops
    value = flops * args.steps * world / (ms * 1e-3) / 1e9
    ba = bytes_alg(A.nnz, A.ncol, st.nnz)
    # dominant kernel (k_numeric, one launch set per phase): A and the
    # phase's B columns read, the phase's C written
    ba_num = st.phases * (A.nnz * 16 + (A.ncol + 1) * 8) + (A.nnz * 16 + (A.ncol + 1) * 8) + \
        st.nnz * 16 + (A.ncol + 1) * 8
    achieved = ba_num / (agg["numeric"] * 1e-3) / 1e9
    out = {
        "metric": metric_name(args.workload, scale, ef),
        "value": value, "unit": "Gmults/s", "ms_per_step": ms / args.steps,
        "spgemm": {"path": "column phases, learned phase sizing (MLP), overflowing columns re-run exactly",
                   "flops": flops, "nnz_c": st.nnz, "phases": st.phases, "max_phase_slots": st.max_phase_nnz,
                   "alloc_over_nnz": st.alloc_nnz / max(st.nnz, 1), "overflow_cols": st.overflow_cols,
                   "overflow_rate": st.overflow_cols / max(A.ncol, 1),
                   "ms_sizing": agg["sizing"], "ms_numeric": agg["numeric"], "ms_rerun": agg["rerun"],
                   "row_checksum": st.row_checksum, "content_hash": f"{st.content_hash:016x}",
                   "val_checksum": st.val_checksum, "bytes_alg": ba,
                   "roofline_frac_whole_step": ba / (ms / args.steps * 1e-3) / 1e9 / hbm,
                   "model": info},
        "exact_two_phase": {"value": flops * args.steps * world / (ms_x * 1e-3) / 1e9, "unit": "Gmults/s",
                            "ms_per_step": ms_x / args.steps, "ms_symbolic": agg_x["sizing"],
                            "ms_numeric": agg_x["numeric"], "phases": st_x.phases,
                            "identical_output": same, "learned_speedup": ms_x / ms},
        "roofline": {"bound": "hbm", "kernel": "k_numeric_x (numeric pass of the big columns, exact fold)",
                     "achieved": achieved, "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": (NUMERIC_DRAM_READ_PER_MULT * flops + NUMERIC_DRAM_WRITE_PER_ENTRY * st.nnz)
                     / max(st.phases, 1),
                     "algorithmic_bytes_per_launch": ba_num / max(st.phases, 1),
                     "traffic_note": "DRAM bytes per launch scaled from profiles/k_numeric_x_s20_cols4096.txt "
                                     "(reads per multiplication, writes per output entry)"},
        "gpu_launches": launches,
        "clocks": ck,
    }
    # ---- e2e: host (pinned) buffers through the public C ABI ---------
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory()

    class _H:
        pass

    def pinned(M):
        H = _H()
        H.nrow, H.ncol = M.nrow, M.ncol
        H.colptr, H.rowidx, H.values = pin(M.colptr).numpy(), pin(M.rowidx).numpy(), pin(M.values).numpy()
        return H

    Ah = pinned(A)
    Bhp = Ah if Bh is A else pinned(Bh)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        st_e = LC.spgemm_phased(Ah, Bhp, max_phase_nnz=budget, ctx=ctx, sizing="learned")
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, "cuda")
    h2d = sum(M.colptr.nbytes + M.rowidx.nbytes + M.values.nbytes for M in (Ah, Bhp))
    d2h = A.ncol * 8 + 3 * 8 * ctx_sms(ctx) * 6 * st_e.phases  # capacities (phase cuts) + checksum partials
    out["e2e"] = {"value": st_e.flops * args.steps * world / e2e_s / 1e9, "unit": "Gmults/s",
                  "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h,
                  "path": "gbc_spgemm_phased (learned sizing) with host pinned A and B: H2D inside the call, "
                          "checksums read back"}
    assert (st_e.nnz, st_e.content_hash) == (st.nnz, st.content_hash)
    model.close()
    return out


def ctx_sms(ctx) -> int:
    import torch

    return torch.cuda.get_device_properties(torch.cuda.current_device()).multi_processor_count


def bench_mcl(ctx):
    """MCL expansion (n = 2^20, 1024 planted clusters, fp32; prune 1e-4,
    select 100): exact two-phase sizing vs learned sizing (network trained
    on another seed), identical output checked."""
    import torch
    from combblas_gb300 import generators as G
    from combblas_gb300 import local as LC
    from combblas_gb300 import mcl as MCL
    from combblas_gb300 import sizing as SZ

    n = 1 << 20
    A = G.mcl_planted(n, 1024, 24.0, 6.0, seed=3)
    At = G.mcl_planted(n, 1024, 24.0, 6.0, seed=4)
    Ad = LC.DeviceMatrix.from_host(A, dtype=np.float32)
    Atd = LC.DeviceMatrix.from_host(At, dtype=np.float32)
    feat, flop, nnz = SZ.features(Atd, Atd, ctx=ctx)
    m = SZ.SizingModel(ctx)
    info = m.fit(feat, nnz, steps=300)
    m.use()
    res = {}
    outs = {}
    for sizing in ("exact", "learned"):
        for _ in range(3):
            R, st = MCL.mcl_expand(Ad, 1e-4, 100, sizing=sizing, ctx=ctx)
            R.free()
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        reps = 5
        for _ in range(reps):
            R, st = MCL.mcl_expand(Ad, 1e-4, 100, sizing=sizing, ctx=ctx)
            if _ < reps - 1:
                R.free()
        torch.cuda.synchronize()
        ms = (time.perf_counter() - t0) / reps * 1e3
        outs[sizing] = R.to_csc()
        R.free()
        res[sizing] = {"ms": ms, "gmults_per_s": st.flops / ms / 1e6, "flops": st.flops, "nnz_c": st.nnz,
                       "ms_symbolic_or_predict": st.ms_symbolic, "ms_numeric": st.ms_numeric,
                       "overflow_cols": st.overflow_cols, "alloc_entries": st.alloc_entries}
    same = all(np.array_equal(x, y) for x, y in zip(outs["exact"], outs["learned"]))
    m.close()
    return {"workload": "MCL expansion n=2^20, 1024 clusters, ~24 intra + ~6 inter nnz/col, fp32, prune 1e-4, top-100",
            "exact": res["exact"], "learned": res["learned"], "identical_output": same,
            "learned_speedup": res["exact"]["ms"] / res["learned"]["ms"],
            "model": {"loss": info["loss"], "margin": info["margin"], "samples": info["samples"],
                      "trained_on": "planted-cluster matrix, seed 4"}}



def bench_spmv(A, ctx, stream, hbm, peak_kind, reps: int = 20):
    """y <- y + A x (PlusTimes fp64) through a plan; HBM roofline of k_spmv."""
    import torch
    from combblas_gb300 import local as LC

    t0 = time.perf_counter()
    plan = LC.SpMVPlan(LC.DeviceMatrix.from_host(A), np.float64, ctx)
    torch.cuda.synchronize()
    build_s = time.perf_counter() - t0
    x = torch.rand(A.ncol, dtype=torch.float64, device="cuda")
    y = torch.zeros(A.nrow, dtype=torch.float64, device="cuda")
    flush = torch.empty(256 << 20, dtype=torch.uint8, device="cuda")  # 256 MB > L2 between runs
    for _ in range(3):
        plan.multiply(x.data_ptr(), y.data_ptr())
    times = []
    for _ in range(reps):
        flush.zero_()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        e0.record(stream)
        plan.multiply(x.data_ptr(), y.data_ptr())
        e1.record(stream)
        torch.cuda.synchronize()
        times.append(e0.elapsed_time(e1))
    ms = float(np.median(times))
    nnz, m, n = A.nnz, A.nrow, A.ncol
    bytes_alg = nnz * (4 + 8) + n * 8 + (m + 1) * 8 + 2 * m * 8
    plan.close()
    return {"op": "y <- y + A x, PlusTimes fp64, R-MAT matrix of this line", "ms": ms,
            "gflops": 2 * nnz / ms / 1e6, "achieved_gbs": bytes_alg / ms / 1e6, "peak": hbm, "peak_kind": peak_kind,
            "frac": bytes_alg / ms / 1e6 / hbm, "bytes_alg": bytes_alg, "plan_build_s": build_s,
            "l2": "256 MB written between runs"}



def bench_msbfs(args, world, A, ctx, stream, hbm, peak_kind, scale, ef):
    """Multi-source BFS from MS_ROOTS seeded roots at once (the masked
    Select2ndMin SpGEMM loop); a step is one whole traversal."""
    import torch
    from combblas_gb300 import _lib
    from combblas_gb300 import bfs as B

    P = A.with_values(None)
    g = B.Graph(P, ctx)
    deg = np.diff(A.colptr)
    roots = np.random.default_rng(SEED + 200).choice(np.nonzero(deg)[0], MS_ROOTS, replace=False)
    par = torch.empty((MS_ROOTS, A.ncol), dtype=torch.int64, device="cuda")
    for _ in range(args.warmup):
        B.msbfs(g, roots, par.data_ptr())
    torch.cuda.synchronize()
    barrier(world)
    clocks = ClockSampler(int(torch.cuda.current_device()))
    clocks.start()
    l0 = _lib.lib().gbc_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    edges = 0
    torch.cuda.nvtx.range_push("timed_msbfs")
    e0.record(stream)
    for _ in range(args.steps):
        _, st = B.msbfs(g, roots, par.data_ptr())
        edges += st.edges
    e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    ms = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
    launches = _lib.lib().gbc_launch_count() - l0
    ck = clocks.stop()
    value = edges * world / (ms * 1e-3) / 1e9
    # expand kernel bytes per traversal: per scanned edge a 4-byte row id, a
    # visited-bit word and a 4-byte candidate read (8-byte frontier entry per
    # (root, vertex)), parents written once per reached pair
    scanned = 2 * st.edges
    bytes_trav = scanned * (4 + 4 + 4) + st.reached * (8 + 8 + 8)
    achieved = bytes_trav / (ms / args.steps * 1e-3) / 1e9
    out = {
        "metric": metric_name(args.workload, scale, ef), "value": value, "unit": "GTEPS",
        "ms_per_step": ms / args.steps, "gpu_launches": launches, "clocks": ck,
        "msbfs": {"roots": MS_ROOTS, "levels": st.levels, "reached_pairs": st.reached, "edges_per_step": st.edges,
                  "loop": "masked Select2ndMin product into a per-(root, vertex) candidate array; one CUDA "
                          "graph per traversal (a conditional while node around the captured level)"},
        "roofline": {"bound": "hbm", "kernel": "k_ms_expand + k_ms_finalize", "achieved": achieved, "peak": hbm,
                     "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm,
                     "traffic": None, "algorithmic_bytes": bytes_trav,
                     "traffic_note": "the level kernels run inside the traversal graph's while node, which ncu "
                                     "does not list as launches; the last level-by-level capture measured "
                                     f"{MSBFS_DRAM_PER_SCANNED_EDGE_LEVEL_REPLAY} DRAM B per scanned edge "
                                     "(profiles/launches_msbfs22.txt)"},
    }
    # e2e: graph upload from host + traversal + parents read back into pinned host memory
    hp = torch.empty((MS_ROOTS, A.ncol), dtype=torch.int64, pin_memory=True)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e_edges = 0
    for _ in range(args.steps):
        g2 = B.Graph(P, ctx)
        st_h = _msbfs_to_host(B, g2, roots, hp)
        e_edges += st_h.edges
        g2.close()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, "cuda")
    out["e2e"] = {"value": e_edges * world / e2e_s / 1e9, "unit": "GTEPS",
                  "h2d_bytes_per_step": int(A.colptr.nbytes + A.rowidx.nbytes + roots.nbytes),
                  "d2h_bytes_per_step": int(hp.numel() * 8),
                  "path": "gbc_graph_create from host CSC + gbc_msbfs writing parents to pinned host memory"}
    assert np.array_equal(hp[:4].numpy(), par[:4].cpu().numpy())
    g.close()
    return out


def _msbfs_to_host(B, g, roots, hp):
    import ctypes as C

    from combblas_gb300 import _lib as L

    roots = np.ascontiguousarray(roots, np.int64)
    st = L.gbc_msbfs_stats()
    L.check(L.lib().gbc_msbfs(g.ctx.h, g.h, roots.ctypes.data, len(roots), C.c_void_p(hp.data_ptr()), L.GBC_HOST,
                              C.byref(st)))
    return st



def bench_batch(args, world, ctx, stream, hbm, peak_kind):
    """The uneven batch: 128 R-MAT A*A (n = 2^10..2^18, edge factor 4..16)
    and 128 Galerkin products R*(A*R^T) (27-point Poisson, side 16..64).
    Batched: products grouped so each group's output fits the device budget,
    each group one gbc_batch (plan, symbolic, one captured graph), Galerkin
    second stages in a batch fed from the first stages' device results.
    One by one: the same products through gbc_spgemm in sequence.  A step is
    the whole set; both arms include symbolic pass and allocation."""
    import torch
    from combblas_gb300 import _lib
    from combblas_gb300 import batch as BT
    from combblas_gb300 import generators as G
    from combblas_gb300 import local as LC

    t0 = time.perf_counter()
    rm, gk = G.batch_c4(256, seed=4)
    log(f"generated the 256-problem batch in {time.perf_counter() - t0:.1f}s")
    dev = lambda M: LC.DeviceMatrix.from_host(M)
    first = [(dev(A), dev(A)) for A in rm] + [(dev(A), dev(Rt)) for A, R, Rt in gk]
    Rs = [dev(R) for A, R, Rt in gk]
    dims = [(A.nrow, Rt.ncol) for A, R, Rt in gk]
    nnz_first = [int(LC._colstats(a, b, ctx)[1].sum()) for a, b in first]
    budget = args.batch_budget_nnz
    groups, cur, acc = [], [], 0
    for p in sorted(range(len(first)), key=lambda q: nnz_first[q]):
        if cur and acc + nnz_first[p] > budget:
            groups.append(cur)
            cur, acc = [], 0
        cur.append(p)
        acc += nnz_first[p]
    groups.append(cur)
    ng = len(rm)

    nnz_second = [0] * len(gk)

    def batched(inputs=None, R_in=None, read_back=False):
        inputs = inputs or first
        flops, d2h = 0, 0
        ars = {}
        for grp in groups:
            b = BT.Batch([inputs[p][0] for p in grp], [inputs[p][1] for p in grp], ctx=ctx)
            flops += b.flops()
            for i, p in enumerate(grp):
                if p >= ng:
                    ars[p - ng] = b.result_device(i, *dims[p - ng])
                if read_back:
                    d2h += b.column_pointers(i).nbytes
            b.close()
        b2 = BT.Batch(R_in or Rs, [ars[q] for q in range(len(gk))], ctx=ctx)
        flops += b2.flops()
        nnz_second[:] = [int(b2.info(q)[1]) for q in range(len(gk))]
        if read_back:
            d2h += sum(b2.column_pointers(q).nbytes for q in range(len(gk)))
        b2.close()
        return flops, d2h

    def one_by_one():
        for p, (a, b) in enumerate(first):
            R = LC.spgemm(a, b, ctx=ctx)
            if p >= ng:
                q = p - ng
                ar = LC.DeviceMatrix(dims[q][0], dims[q][1], *result_to_torch(R))
                R2 = LC.spgemm(Rs[q], ar, ctx=ctx)
                R2.free()
            R.free()

    for _ in range(args.warmup):
        batched()
    one_by_one()
    first_host = [(A, A) for A in rm] + [(A, Rt) for A, R, Rt in gk]
    Rs_host = [R for A, R, Rt in gk]
    torch.cuda.synchronize()
    clocks = ClockSampler(int(torch.cuda.current_device()))
    clocks.start()
    l0 = _lib.lib().gbc_launch_count()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    torch.cuda.nvtx.range_push("timed_batch")
    e0.record(stream)
    for _ in range(args.steps):
        flops, _ = batched()
    e1.record(stream)
    torch.cuda.synchronize()
    torch.cuda.nvtx.range_pop()
    ms = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
    launches = _lib.lib().gbc_launch_count() - l0
    ck = clocks.stop()
    e0.record(stream)
    for _ in range(args.steps):
        one_by_one()
    e1.record(stream)
    torch.cuda.synchronize()
    ms_1 = max_over_ranks(e0.elapsed_time(e1), world, "cuda")
    # e2e: first-stage inputs from host memory (copied inside gbc_batch_create),
    # every product's column pointers read back
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        _, d2h = batched(first_host, Rs_host, read_back=True)
    torch.cuda.synchronize()
    e2e_s = max_over_ranks(time.perf_counter() - t0, world, "cuda")
    h2d = sum(M.colptr.nbytes + M.rowidx.nbytes + M.values.nbytes for pair in first_host for M in pair) + \
        sum(M.colptr.nbytes + M.rowidx.nbytes + M.values.nbytes for M in Rs_host)
    # algorithmic bytes of one step: every product reads its operands once and
    # writes its output (16 B per entry + column pointers)
    csc_bytes = lambda M: M.colptr.nbytes + M.rowidx.nbytes + M.values.nbytes
    ba = sum(csc_bytes(a) + csc_bytes(b) + 16 * nz + 8 * (b.ncol + 1) for (a, b), nz in zip(first_host, nnz_first))
    ba += sum(csc_bytes(R) + 16 * nz_ar + 8 * (dims[q][1] + 1) + 16 * nz2 + 8 * (dims[q][1] + 1)
              for q, (R, nz_ar, nz2) in enumerate(zip(Rs_host, nnz_first[ng:], nnz_second)))
    achieved = ba / (ms / args.steps * 1e-3) / 1e9
    result_sets = (rm, gk)
    return {
        "e2e": {"value": flops * args.steps * world / e2e_s / 1e9, "unit": "Gmults/s", "h2d_bytes_per_step": h2d,
                "d2h_bytes_per_step": d2h,
                "path": "gbc_batch_create from host CSC arrays + gbc_batch_run; column pointers of every product "
                        "read back (the products stay on the device)"},
        "metric": metric_name(args.workload, 0, 0), "value": flops * args.steps * world / (ms * 1e-3) / 1e9,
        "unit": "Gmults/s", "ms_per_step": ms / args.steps, "gpu_launches": launches, "clocks": ck,
        "batch": {"problems": 256, "groups": len(groups), "budget_nnz": budget, "flops": flops,
                  "one_by_one_gmults": flops * args.steps / (ms_1 * 1e-3) / 1e9,
                  "one_by_one_ms_per_step": ms_1 / args.steps, "batched_speedup": ms_1 / ms},
        "roofline": {"bound": "hbm", "kernel": "whole batched step (every pass of every product)",
                     "achieved": achieved, "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": achieved / hbm, "algorithmic_bytes": ba, "traffic": None,
                     "note": "operands read once and outputs written once per product (16 B per entry)"},
        "_problems": result_sets,
    }


# ------------------------------------------- every configuration, one line
def _timed(stream, fn, reps):
    """Device time of `reps` calls of fn (CUDA events on `stream`), ms per call."""
    import torch

    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(reps):
        fn()
    e1.record(stream)
    torch.cuda.synchronize()
    return e0.elapsed_time(e1) / reps


def _pinned_result_buffers(R):
    """Pinned host arrays for a result's cp, jc, ir and values."""
    import torch

    vt = torch.float64 if np.dtype(R.dtype) == np.float64 else torch.float32
    return [torch.empty(max(n, 1), dtype=t).pin_memory()
            for n, t in ((R.nzc + 1, torch.int64), (R.nzc, torch.int64), (R.nnz, torch.int64), (R.nnz, vt))]


def _same(a, b):
    """Bit-exact equality of (colptr, rows, values) triples."""
    return all(np.array_equal(np.asarray(x).view(np.int64) if np.asarray(x).dtype == np.float64 else x,
                              np.asarray(y).view(np.int64) if np.asarray(y).dtype == np.float64 else y)
               for x, y in zip(a, b))


def parity_spgemm_sample(A, Ad, ctx, ncols=4096):
    """The scale-20 product on a seeded sample of B columns (the full row
    range) against the oracle, under both folds: bit-exact."""
    import oracle as O
    from combblas_gb300 import local as LC

    Bh, cols = column_sample(A, ncols / A.ncol, seed=11)
    Bd = LC.DeviceMatrix.from_host(Bh)
    out = {"columns": len(cols), "check": "bit-exact (pattern and value bits) against oracle/oracle.c"}
    for fold in ("exact", "ordered"):
        R = LC.spgemm(Ad, Bd, ctx=ctx, fold=fold)
        got = R.to_csc()
        R.free()
        (pcp, prow, pval), (flop, _) = O.port_spgemm(A, Bh, O.SR_PLUSTIMES_F64, fold=fold, want_counts=True)
        out[f"{fold}_fold"] = bool(_same(got, (pcp, prow, pval)))
        out["mults"] = int(flop.sum())
        out["entries"] = int(len(prow))
        if fold == "exact":
            xv = pval
        else:
            out["max_rel_exact_vs_hash_order"] = float(np.max(np.abs(xv - pval) / np.abs(pval))) if len(pval) else 0.0
    out["ok"] = out["exact_fold"] and out["ordered_fold"]
    return out


def bench_c1(args, ctx, stream, hbm, peak_kind):
    """C1: C = A*A on the scale-14 R-MAT (ef 8), PlusTimes fp64, exact
    two-phase, device-resident inputs; the whole product is checked."""
    import torch
    import oracle as O
    from combblas_gb300 import generators as G
    from combblas_gb300 import local as LC

    A = G.rmat(14, 8, seed=SEED)
    Ad = LC.DeviceMatrix.from_host(A)
    reps = max(args.steps, 5)
    for _ in range(3):
        LC.spgemm(Ad, Ad, ctx=ctx).free()
    st = {}

    def one():
        R = LC.spgemm(Ad, Ad, ctx=ctx)
        st["s"] = R.stats
        R.free()

    ms = _timed(stream, one, reps)
    s0 = st["s"]
    got = LC.spgemm(Ad, Ad, ctx=ctx).to_csc()
    t0 = time.perf_counter()
    (pcp, prow, pval), (flop, _) = O.port_spgemm(A, A, O.SR_PLUSTIMES_F64, want_counts=True)
    cpu_s = time.perf_counter() - t0
    exact_ok = _same(got, O.port_spgemm(A, A, O.SR_PLUSTIMES_F64, fold="exact"))
    ordered_ok = _same(LC.spgemm(Ad, Ad, ctx=ctx, fold="ordered").to_csc(), (pcp, prow, pval))
    ba = bytes_alg(A.nnz, A.ncol, s0.nnz)
    # e2e: host CSC in (pinned), the whole product read back into pinned
    # host arrays (allocated once, like the caller's output buffers)
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    Ah = G.CSC(A.nrow, A.ncol, pin(A.colptr), pin(A.rowidx), pin(A.values))
    R = LC.spgemm(Ah, Ah, ctx=ctx)
    outs = _pinned_result_buffers(R)
    R.free()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        R = LC.spgemm(Ah, Ah, ctx=ctx)
        R.copy_to(*[o.data_ptr() for o in outs])
        R.free()
    e2e_s = (time.perf_counter() - t0) / reps
    d2h = sum(o.numel() * o.element_size() for o in outs)
    return {
        "workload": "R-MAT s14 ef8 A*A, PlusTimes fp64 (exact fold), exact two-phase, inputs resident",
        "value": s0.flops / (ms * 1e-3) / 1e9, "unit": "Gmults/s", "ms_per_step": ms, "flops": s0.flops,
        "nnz_c": s0.nnz, "ms_symbolic": s0.ms_symbolic, "ms_numeric": s0.ms_numeric,
        "roofline": {"bound": "hbm", "kernel": "whole product (symbolic + numeric kernels)",
                     "achieved": ba / (ms * 1e-3) / 1e9, "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": ba / (ms * 1e-3) / 1e9 / hbm, "algorithmic_bytes": ba, "traffic": None},
        "cpu_baseline": {"value": int(flop.sum()) / cpu_s / 1e9, "unit": "Gmults/s", "cores": O.port_num_threads(),
                         "kind": "port", "sample": "the whole product (oracle/oracle.c, the reference's hash path)"},
        "e2e": {"value": s0.flops / e2e_s / 1e9, "unit": "Gmults/s",
                "h2d_bytes_per_step": int(2 * (A.colptr.nbytes + A.rowidx.nbytes + A.values.nbytes)),
                "d2h_bytes_per_step": int(d2h),
                "path": "gbc_spgemm with pinned host CSC inputs, the product (cp, jc, ir, num) copied back "
                        "into pinned host arrays"},
        "parity": {"ok": bool(exact_ok and ordered_ok), "exact_fold_vs_oracle": bool(exact_ok),
                   "ordered_fold_vs_oracle": bool(ordered_ok), "check": "whole product, bit-exact"},
    }


def bench_c2(args, A, ctx, stream, hbm, peak_kind, world):
    """C2: BFS on the scale-20 R-MAT from 64 seeded roots, top-down only
    (the configuration's algorithm) and direction-optimizing; parents and
    levels of 4 roots checked against the oracle."""
    import torch
    import oracle as O
    from combblas_gb300 import _lib
    from combblas_gb300 import bfs as B
    from combblas_gb300 import generators as G

    P = A.with_values(None)
    g = B.Graph(P, ctx)
    par = torch.empty(A.ncol, dtype=torch.int64, device="cuda")
    lev = torch.empty(A.ncol, dtype=torch.int64, device="cuda")
    roots = bfs_roots(A)
    res = {}
    for policy in ("topdown", "auto"):
        g.set_policy(policy)
        for r in roots[:3]:
            B.bfs_device(g, int(r), par.data_ptr(), lev.data_ptr())
        edges = [0]
        l0 = _lib.lib().gbc_launch_count()

        def run():
            for r in roots:
                edges[0] += B.bfs_device(g, int(r), par.data_ptr(), lev.data_ptr()).edges

        ms = _timed(stream, run, 1)
        res[policy] = {"gteps": edges[0] / (ms * 1e-3) / 1e9, "ms_64_roots": ms, "edges": edges[0],
                       "gpu_launches": _lib.lib().gbc_launch_count() - l0}
    g.set_policy("topdown")
    ok = True
    for r in roots[:4]:
        p1, l1, _ = B.bfs(g, int(r))
        p2, l2, _ = O.port_bfs(P, int(r))
        ok = ok and np.array_equal(p1, p2) and np.array_equal(l1, l2)
    g.close()
    # e2e, as the reference's BFS benchmark runs: the graph uploaded once
    # from pinned host CSC, then every root's parents and levels written
    # into pinned host arrays (gbc_bfs with GBC_HOST)
    import ctypes as C

    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    Ph = G.CSC(A.nrow, A.ncol, pin(A.colptr), pin(A.rowidx), None)
    hpar = torch.empty(A.ncol, dtype=torch.int64).pin_memory()
    hlev = torch.empty(A.ncol, dtype=torch.int64).pin_memory()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    e_edges = 0
    g2 = B.Graph(Ph, ctx)
    g2.set_policy("topdown")
    for r in roots:
        st_h = _lib.gbc_bfs_stats()
        _lib.check(_lib.lib().gbc_bfs(ctx.h, g2.h, int(r), C.c_void_p(hpar.data_ptr()), C.c_void_p(hlev.data_ptr()),
                                      C.byref(st_h), _lib.GBC_HOST))
        e_edges += st_h.edges
    g2.close()
    e2e_s = time.perf_counter() - t0
    ok = ok and np.array_equal(hpar.numpy(), B.bfs(P, int(roots[-1]), ctx=ctx)[0])
    v, desc, th = cpu_bfs_rate(A, roots[:8], 10.0)
    td = res["topdown"]
    bytes_td = td["edges"] * 2 * 4 + len(roots) * A.ncol * 16
    return {
        "workload": "BFS R-MAT s20 ef16, 64 roots, SelectMin parents; value = top-down only",
        "value": td["gteps"] * world, "unit": "GTEPS", "topdown": td, "direction_optimizing": res["auto"],
        "roofline": {"bound": "hbm", "kernel": "k_bfs_td (top-down levels)", "achieved": bytes_td / (td["ms_64_roots"] * 1e-3) / 1e9,
                     "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": bytes_td / (td["ms_64_roots"] * 1e-3) / 1e9 / hbm, "traffic": None,
                     "algorithmic_bytes": bytes_td,
                     "note": "4 B per scanned edge (each undirected edge scanned twice) + 16 B parent/level per vertex"},
        "cpu_baseline": {"value": v, "unit": "GTEPS", "cores": th, "kind": "port", "sample": desc},
        "e2e": {"value": e_edges / e2e_s / 1e9, "unit": "GTEPS", "h2d_bytes_per_step": int(A.colptr.nbytes + A.rowidx.nbytes),
                "d2h_bytes_per_step": len(roots) * 2 * A.ncol * 8,
                "path": "gbc_graph_create from pinned host CSC once, then gbc_bfs (top-down) for each of the 64 roots "
                        "writing parents and levels into pinned host arrays"},
        "parity": {"ok": bool(ok), "roots": 4, "check": "parents and levels bit-exact against the oracle's BFS"},
    }


def bench_c3(ctx, hbm, peak_kind):
    """C3: MCL expansion step (n = 2^20 planted clusters, fp32): exact vs
    learned sizing (bench_mcl), plus roofline, CPU baseline, e2e and the
    whole selected product against the oracle."""
    import torch
    import oracle as O
    from combblas_gb300 import generators as G
    from combblas_gb300 import mcl as MCL

    out = bench_mcl(ctx)
    n = 1 << 20
    A = G.mcl_planted(n, 1024, 24.0, 6.0, seed=3)
    R, st = MCL.mcl_expand(A, 1e-4, 100, ctx=ctx)
    got = R.to_csc()
    R.free()
    t0 = time.perf_counter()
    (pcp, prow, pval), (flop, _) = O.port_spgemm(A, A, O.SR_PLUSTIMES_F32, sorted=False, want_counts=True)
    scp, srow, sval = O.port_mcl_select(pcp, prow, pval, 1e-4, 100)
    cpu_s = time.perf_counter() - t0
    exp = O.canonical_csc(scp, srow, sval)
    ok = all(np.array_equal(x, y) for x, y in zip(got, exp))
    # e2e: the host matrix in (pinned), the selected product back into
    # pinned host arrays
    pin = lambda a: torch.from_numpy(np.ascontiguousarray(a)).pin_memory().numpy()
    Ap = G.CSC(A.nrow, A.ncol, pin(A.colptr), pin(A.rowidx), pin(np.asarray(A.values, np.float32)))
    R, st_e = MCL.mcl_expand(Ap, 1e-4, 100, ctx=ctx)
    outs = _pinned_result_buffers(R)
    R.free()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    reps = 3
    for _ in range(reps):
        R, st_e = MCL.mcl_expand(Ap, 1e-4, 100, ctx=ctx)
        R.copy_to(*[o.data_ptr() for o in outs])
        R.free()
    e2e_s = (time.perf_counter() - t0) / reps
    d2h = sum(o.numel() * o.element_size() for o in outs)
    ex = out["exact"]
    nnz_sel = len(exp[1])
    ba = 2 * (A.nnz * 12 + (n + 1) * 8) + ex["nnz_c"] * 12 + ex["nnz_c"] * 12 + nnz_sel * 12
    out.update({
        "value": ex["gmults_per_s"], "unit": "Gmults/s",
        "roofline": {"bound": "hbm", "kernel": "expansion + prune/select (whole step, exact sizing)",
                     "achieved": ba / (ex["ms"] * 1e-3) / 1e9, "peak": hbm, "peak_kind": peak_kind, "unit": "GB/s",
                     "frac": ba / (ex["ms"] * 1e-3) / 1e9 / hbm, "algorithmic_bytes": ba, "traffic": None,
                     "note": "A read twice, C written and read once, selected entries written (12 B per entry)"},
        "cpu_baseline": {"value": int(flop.sum()) / cpu_s / 1e9, "unit": "Gmults/s", "cores": O.port_num_threads(),
                         "kind": "port", "sample": "the whole step (hash-path product + MCLPruneRecoverySelect restatement)"},
        "e2e": {"value": st_e.flops / e2e_s / 1e9, "unit": "Gmults/s",
                "h2d_bytes_per_step": int(A.colptr.nbytes + A.rowidx.nbytes + A.values.nbytes),
                "d2h_bytes_per_step": int(d2h),
                "path": "gbc_mcl_expand_recover_f32 from pinned host CSC, the selected product (cp, jc, ir, num) "
                        "copied back into pinned host arrays"},
        "parity": {"ok": bool(ok), "check": "the whole selected product bit-exact against the oracle "
                                            "(PlusTimes fp32 product in hash order + prune/select)"},
    })
    return out


def parity_batch(rm, gk, ctx, nprob=16):
    """16 of the 256 batch problems (the first R-MAT and Galerkin ones by a
    seeded choice) through a batch, against the oracle's exact fold."""
    import oracle as O
    from combblas_gb300 import batch as BT

    rng = np.random.default_rng(SEED + 300)
    pick_r = sorted(rng.choice(len(rm), nprob // 2, replace=False).tolist())
    pick_g = sorted(rng.choice(len(gk), nprob // 2, replace=False).tolist())
    As = [rm[p] for p in pick_r] + [gk[q][0] for q in pick_g]
    Bs = [rm[p] for p in pick_r] + [gk[q][2] for q in pick_g]
    b = BT.Batch(As, Bs, ctx=ctx)
    ok = True
    for i, (A, B) in enumerate(zip(As, Bs)):
        ok = ok and _same(b.result(i), O.port_spgemm(A, B, O.SR_PLUSTIMES_F64, fold="exact"))
    b.close()
    return {"ok": bool(ok), "problems": nprob, "check": "first-stage products through one batch, bit-exact "
                                                        "against the oracle's exact fold"}


def parity_msbfs(A, ctx, roots):
    """Parent rows of 2 roots of the multi-source traversal against the
    oracle's single-source BFS (min-parent semantics)."""
    import oracle as O
    from combblas_gb300 import bfs as B

    P = A.with_values(None)
    g = B.Graph(P, ctx)
    par, _ = B.msbfs(g, roots[:2])
    g.close()
    ok = True
    for i in range(2):
        p2, _, _ = O.port_bfs(P, int(roots[i]))
        other = np.arange(A.ncol) != int(roots[i])
        ok = ok and par[i][int(roots[i])] == int(roots[i]) and np.array_equal(np.asarray(par[i])[other], p2[other])
    return {"ok": bool(ok), "roots": 2,
            "check": "parent rows bit-exact against the oracle's single-source BFS (min parent); the root's own "
                     "entry is the root (sources start visited in the multi-source loop)"}


def result_to_torch(R):
    """(cp, ir, num) device copies of a product (CSC over the stored columns
    of B), to feed a second product."""
    import torch

    t_cp = torch.empty(R.nzc + 1, dtype=torch.int64, device="cuda")
    t_ir = torch.empty(max(R.nnz, 1), dtype=torch.int64, device="cuda")
    t_num = torch.empty(max(R.nnz, 1), dtype=torch.float64, device="cuda")
    R.copy_to(t_cp.data_ptr(), None, t_ir.data_ptr(), t_num.data_ptr(), where=1)
    return t_cp, t_ir[:R.nnz], t_num[:R.nnz]



# ------------------------------------------------------------------- ours
def run_ours(args, world, rank, local):
    import torch

    torch.cuda.set_device(local)
    from combblas_gb300 import _lib
    from combblas_gb300 import bfs as B
    from combblas_gb300 import local as LC

    ctx = LC.Context(local)
    stream = torch.cuda.current_stream()
    ctx.set_stream(stream.cuda_stream)
    hbm, peak_kind = peaks()
    result: dict = {}
    if args.workload == "batch256":
        A, scale, ef = None, 0, 0
        result.update(bench_batch(args, world, ctx, stream, hbm, peak_kind))
    else:
        A, scale, ef = make_graph(args.workload, args.scale)
        Ad = LC.DeviceMatrix.from_host(A)
        torch.cuda.synchronize()

    # ---- SpGEMM, inputs resident in HBM -------------------------------
    every = args.workload == "spgemm20" and not args.headline_only  # every configuration in this line
    if args.workload.startswith("spgemm"):
        result.update(bench_spgemm(args, world, A, Ad, ctx, stream, scale, ef, hbm, peak_kind))
        if not args.no_mcl and world >= 1 and not every:
            result["mcl"] = bench_mcl(ctx)

    if args.workload == "msbfs22":
        result.update(bench_msbfs(args, world, A, ctx, stream, hbm, peak_kind, scale, ef))

    # ---- dense-vector SpMV on the same matrix (dcsc_gespmv) ---------------
    if args.workload.startswith("spgemm") and not args.no_bfs:
        result["spmv"] = bench_spmv(A, ctx, stream, hbm, peak_kind)

    # ---- BFS: 64 roots, level loop as a replayed CUDA graph --------------
    if args.workload == "bfs20" or (args.workload.startswith("spgemm") and not args.no_bfs and not every):
        g = B.Graph(A.with_values(None), ctx)
        par = torch.empty(A.ncol, dtype=torch.int64, device="cuda")
        lev = torch.empty(A.ncol, dtype=torch.int64, device="cuda")
        roots = bfs_roots(A)
        for r in roots[:3]:
            B.bfs_device(g, int(r), par.data_ptr(), lev.data_ptr())
        torch.cuda.synchronize()
        edges = 0
        l0 = _lib.lib().gbc_launch_count()
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        if args.workload == "bfs20":
            clocks = ClockSampler(local)
            clocks.start()
        torch.cuda.nvtx.range_push("timed_bfs")
        e0.record(stream)
        for r in roots:
            st_b = B.bfs_device(g, int(r), par.data_ptr(), lev.data_ptr())
            edges += st_b.edges
        e1.record(stream)
        torch.cuda.synchronize()
        torch.cuda.nvtx.range_pop()
        bfs_ms = e0.elapsed_time(e1)
        gteps = edges / (bfs_ms * 1e-3) / 1e9
        bfs_launches = _lib.lib().gbc_launch_count() - l0
        result["bfs"] = {"gteps": gteps, "roots": len(roots), "ms_total": bfs_ms, "edges": edges,
                         "semiring": "SelectMin (min parent)",
                         "loop": "one CUDA graph per traversal: a conditional while node around the captured level"}
        if args.workload == "bfs20":
            result.update({"metric": metric_name(args.workload, scale, ef), "value": gteps * world,
                           "unit": "GTEPS", "ms_per_step": bfs_ms / len(roots), "gpu_launches": bfs_launches,
                           "clocks": clocks.stop()})
            # e2e: host graph upload each step
            t0 = time.perf_counter()
            P = A.with_values(None)
            e_edges = 0
            for r in roots[:8]:
                par_h, lev_h, st_h = B.bfs(P, int(r), ctx=ctx)
                e_edges += st_h.edges
            e2e_s = time.perf_counter() - t0
            result["e2e"] = {"value": e_edges / e2e_s / 1e9, "unit": "GTEPS",
                             "h2d_bytes_per_step": (A.colptr.nbytes + A.rowidx.nbytes),
                             "d2h_bytes_per_step": 2 * A.ncol * 8}
            achieved = edges * 2 * 4 / (bfs_ms * 1e-3) / 1e9
            result["roofline"] = {"bound": "hbm", "kernel": "k_bfs_td + k_bfs_bu", "achieved": achieved, "peak": hbm,
                                  "peak_kind": peak_kind, "unit": "GB/s", "frac": achieved / hbm, "traffic": None}

    # ---- the other configurations, each with its own roofline, CPU
    # baseline, e2e and parity check; parity of the headline on a column
    # sample of the full-size product ------------------------------------
    if every:
        import types

        import torch

        sub = types.SimpleNamespace(**vars(args))
        sub.steps, sub.warmup = min(args.steps, 3), 1
        cfg = {}
        parity = {"spgemm20_sample": parity_spgemm_sample(A, Ad, ctx)}
        log("parity s20 sample:", parity["spgemm20_sample"])
        cfg["C1_spgemm14"] = bench_c1(sub, ctx, stream, hbm, peak_kind)
        cfg["C2_bfs20"] = bench_c2(sub, A, ctx, stream, hbm, peak_kind, world)
        if not args.no_mcl:
            cfg["C3_mcl20"] = bench_c3(ctx, hbm, peak_kind)
        if not args.no_bfs:
            spmv = bench_spmv(A, ctx, stream, hbm, peak_kind)
            result["spmv"] = spmv
        del Ad
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        # C4: the uneven batch
        c4 = bench_batch(sub, world, ctx, stream, hbm, peak_kind)
        rm4, gk4 = c4.pop("_problems")
        v, desc, th = cpu_batch_rate(8.0)
        c4 = {"workload": metric_name("batch256", 0, 0), "value": c4["value"], "unit": c4["unit"], "ms_per_step": c4["ms_per_step"],
              "batch": c4["batch"], "roofline": c4["roofline"], "e2e": c4["e2e"], "gpu_launches": c4["gpu_launches"],
              "cpu_baseline": {"value": v, "unit": "Gmults/s", "cores": th, "kind": "port", "sample": desc},
              "parity": parity_batch(rm4, gk4, ctx)}
        cfg["C4_batch256"] = c4
        del rm4, gk4
        torch.cuda.synchronize()
        torch.cuda.empty_cache()
        # C5: multi-source BFS on scale 22
        A22, s22, e22 = make_graph("msbfs22")
        c5 = bench_msbfs(sub, world, A22, ctx, stream, hbm, peak_kind, s22, e22)
        roots22 = np.random.default_rng(SEED + 200).choice(np.nonzero(np.diff(A22.colptr))[0], MS_ROOTS,
                                                           replace=False)
        v, desc, th = cpu_bfs_rate(A22, roots22[:2], 10.0)
        cfg["C5_msbfs22"] = {"workload": metric_name("msbfs22", s22, e22), "value": c5["value"], "unit": "GTEPS",
                             "ms_per_step": c5["ms_per_step"], "msbfs": c5["msbfs"], "roofline": c5["roofline"],
                             "e2e": c5["e2e"], "gpu_launches": c5["gpu_launches"],
                             "cpu_baseline": {"value": v, "unit": "GTEPS", "cores": th, "kind": "port",
                                              "sample": desc + " (single-source BFS of the oracle; the multi-source "
                                                               "loop does the same work per root)"},
                             "parity": parity_msbfs(A22, ctx, roots22)}
        del A22
        for k, c in cfg.items():
            parity[k] = c["parity"]["ok"]
        parity["all_ok"] = bool(parity["spgemm20_sample"]["ok"] and all(c["parity"]["ok"] for c in cfg.values()))
        result["configs"] = cfg
        result["parity"] = parity

    # ---- CPU baseline (rank 0, N=1 only) -------------------------------
    if rank == 0 and world == 1 and not args.no_cpu:
        if args.workload == "batch256":
            v, desc, th = cpu_batch_rate(15.0)
            result["cpu_baseline"] = {"value": v, "unit": "Gmults/s", "cores": th, "kind": "port", "sample": desc}
        elif args.workload in ("bfs20", "msbfs22"):
            v, desc, th = cpu_bfs_rate(A, bfs_roots(A)[:8], 15.0)
            result["cpu_baseline"] = {"value": v, "unit": "GTEPS", "cores": th, "kind": "port",
                                      "sample": desc + " (single-source BFS of the oracle's C restatement; the "
                                                       "multi-source loop does the same work per root)"
                                      if args.workload == "msbfs22" else desc}
        else:
            v, desc, th = cpu_spgemm_rate(A, 15.0)
            result["cpu_baseline"] = {"value": v, "unit": "Gmults/s", "cores": th, "kind": "port",
                                      "sample": desc + " (oracle/oracle.c: the reference's hash-path algorithm)",
                                      "calibration": CPU_CALIBRATION}
    line = {
        "metric": result["metric"], "value": result["value"], "unit": result["unit"], "n_gpus": world,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": result["ms_per_step"], "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None,
        "dtype": "f64" if args.workload.startswith("spgemm") or args.workload == "batch256" else "int64",
        "data": "synthetic (seeded R-MAT, numpy generator)",
        "config": workload_config(args, scale, ef, world),
    }
    for k in ("roofline", "cpu_baseline", "e2e", "gpu_launches", "clocks", "spgemm", "exact_two_phase", "mcl", "bfs",
              "msbfs", "batch", "spmv", "parity", "configs"):
        if k in result:
            line[k] = result[k]
    if rank == 0:
        print(json.dumps(line), flush=True)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--workload", choices=["spgemm20", "bfs20", "spgemm14", "msbfs22", "batch256"],
                    default="spgemm20")
    ap.add_argument("--phase-nnz", type=int, default=3 << 30)
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-mcl", action="store_true", help="skip the MCL exact-vs-learned comparison")
    ap.add_argument("--no-bfs", action="store_true", help="skip the BFS sub-measurement of SpGEMM workloads")
    ap.add_argument("--scale", type=int, default=0, help="override the R-MAT scale (profiling runs)")
    ap.add_argument("--batch-budget-nnz", type=int, default=6 << 30,
                    help="batch256: output entries one batch group may hold")
    ap.add_argument("--headline-only", action="store_true",
                    help="spgemm20: only the headline product (not the other configurations and parity checks)")
    ap.add_argument("--bcols", type=int, default=0,
                    help="profiling case: B = A(:, this many seeded random columns) instead of A")
    args = ap.parse_args()
    args.warmup = max(args.warmup, 3) if args.impl == "ours" else args.warmup
    world, rank, local = dist_setup(args)
    if args.impl == "reference":
        run_reference(args, world, rank)
    else:
        if not os.path.exists(os.path.join(ROOT, "combblas_gb300", "libgbcomb.so")):
            from combblas_gb300 import build as BLD

            BLD.build()
        run_ours(args, world, rank, local)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


if __name__ == "__main__":
    main()
