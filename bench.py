#!/usr/bin/env python
"""Benchmark: batched uneven steady VLM solves on GB300.

Workload (one step): 512 seeded trapezoidal half wings (nc ~ U{4..32},
ns ~ U{4..64}, AR ~ U[4,12], taper ~ U[0.3,1], sweep ~ U[0,35] deg, numpy
PCG64 seed 20261203) with 8 angles of attack each (U[-8,8] deg) = 4096
solves; every solve yields gamma, CL, CDi and CM.  ``--mode shared`` (the
default) builds one AIC per wing at alpha = 0 and solves the 8 angles as
right-hand sides; ``--mode exact`` builds one AIC per wing and angle with
the reference's alpha-dependent collocation points and wake.

``value`` is solves/s with inputs resident on the device: K steps, each one
replay of a step's CUDA graph, with ``--in-flight`` (default 2) batches in
flight on their own streams (BatchPipeline: the next batch's assembly and
small systems fill the SMs that the current batch's largest factorisations
leave idle), timed with CUDA events from the launching stream over all of
them; the AIC set is larger than L2, so no flush is needed.  The
``one_in_flight`` record gives the same with one batch at a time.  ``e2e``
times the same through the public API with host buffers: H2D of the packed
vertices and angles from pinned memory, the graph, and D2H of the
coefficients and every gamma, per batch, with the next batch submitted
before the current one is collected.  ``cpu_baseline`` times the CPU restatement of the reference
backend (float, all host threads) on a bounded sample of the same cases.

``--impl reference`` times only that CPU implementation and prints its own
line.  Under torchrun each rank runs its own replica (replicas only: the
path has no exchange step); rank 0 prints.
"""
import argparse
import json
import math
import os
import subprocess
import sys
import threading
import time

import numpy as np

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "solves/s + p99 latency, batched/served vs plain on 1 GB300 at CL err≤1e-5"
SEED = 20261203
FLOP_PER_INTERACTION = 558  # Biot-Savart ring-point interaction, counted from the reference kernel


def parse():
    p = argparse.ArgumentParser()
    p.add_argument("--gpus", type=int, default=1)
    p.add_argument("--steps", type=int, default=60)
    p.add_argument("--warmup", type=int, default=3)
    p.add_argument("--impl", default="gb300", choices=["gb300", "reference"])
    p.add_argument("--mode", default="shared", choices=["shared", "exact"])
    p.add_argument("--cases", type=int, default=512)
    p.add_argument("--alphas", type=int, default=8)
    p.add_argument("--refine", type=int, default=1,
                   help="refinement sweeps (double residual); 1 keeps every solve of the batch within CL/CM 1e-5")
    p.add_argument("--fp64-residual", action="store_true",
                   help="refinement residual of the FP64 system (float AIC plus its float-pair correction)")
    p.add_argument("--cpu-seconds", type=float, default=15.0)
    p.add_argument("--ref-step-seconds", type=float, default=2.5,
                   help="reference arm: CPU time one step's fixed subset of the batch is sized to")
    p.add_argument("--no-cpu-baseline", action="store_true")
    p.add_argument("--no-configs", action="store_true",
                   help="skip the short records of configurations A, B, C, E and the exact formulation")
    p.add_argument("--plain-solves", type=int, default=48)
    p.add_argument("--in-flight", type=int, default=2,
                   help="batches in flight (BatchPipeline depth) for the headline and its end-to-end number; "
                        "the one-in-flight rate and latency are reported beside them")
    p.add_argument("--workload", default="batch", choices=["batch", "large", "uvlm", "served", "aero2dof", "nlvlm", "hbvlm"],
                   help="batch: the headline batched workload; large: one 128x128 elliptic wing, 64 alphas; "
                        "uvlm: 20x80 rectangular wing, 500 pitch-plunge steps")
    p.add_argument("--uvlm-steps", type=int, default=500)
    p.add_argument("--rates", default="2,8,32", help="served: Poisson arrival rates (requests/s) to sweep")
    p.add_argument("--requests", type=int, default=45, help="served: requests per rate")
    p.add_argument("--rollup", type=int, default=1)
    p.add_argument("--large-n", type=int, default=128, help="large: chordwise = spanwise panels of the elliptic wing")
    p.add_argument("--large-geometry", default="reference", choices=["reference", "generated"],
                   help="large: the reference's elliptic mesh (tip chord 0.0707) or the zero-tip-chord analytic one")
    return p.parse_args()


def max_over_ranks(x, world, device):
    """The largest of every rank's x (all ranks get it): the slowest replica's time."""
    if world == 1:
        return x
    import torch
    import torch.distributed as dist
    t = torch.tensor([x], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def replica_value(units_per_rank, world, ms):
    """Whole-job throughput of independent replicas: every rank's units over the slowest rank's time."""
    return units_per_rank * world / (ms / 1000.0)


def dist_env():
    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return rank, world, local


def workload(args):
    from tinyvlm_gb300 import mesh as M
    return M.batch_cases(args.cases, seed=SEED, n_alpha=args.alphas)


def config(args, cases):
    n = [c.n for c in cases]
    return {"workload": "batched steady VLM: %d trapezoidal half wings x %d alpha, %s AIC" %
                        (len(cases), args.alphas, "shared" if args.mode == "shared" else "per-alpha"),
            "cases": len(cases), "alphas_per_case": args.alphas, "mode": args.mode,
            "panels_min": int(min(n)), "panels_max": int(max(n)), "panels_sum": int(sum(n)),
            "seed": SEED, "refine_iters": args.refine, "fp64_residual": bool(args.fp64_residual),
            "l2": "not flushed: the step's AIC set is larger than the 129 MB L2"}


# ---------------------------------------------------------------------------
# CPU side: the oracle port of the reference backend, float, all threads
# ---------------------------------------------------------------------------
def stratified_order(cases):
    """Case indices such that every prefix samples the batch's panel counts
    evenly: the cases sorted by size, visited in van der Corput (base 2)
    order, so a CPU sample of a few cases has the whole batch's size mix."""
    by_size = sorted(range(len(cases)), key=lambda i: cases[i].n)
    n, out, seen, k = len(cases), [], set(), 0
    while len(out) < n:
        x, f, q = 0.0, 0.5, k
        while q:
            x += f * (q & 1)
            q >>= 1
            f *= 0.5
        i = by_size[min(n - 1, int(x * n))]
        if i not in seen:
            seen.add(i)
            out.append(i)
        k += 1
        if k > 64 * n:  # every remaining index, in size order
            out += [j for j in by_size if j not in seen]
            break
    return out


def cpu_sample(args, cases, seconds):
    from oracle import oracle as O
    O.lib()
    threads = O.num_threads()
    done, t0 = 0, time.perf_counter()
    used = 0
    order = stratified_order(cases)
    for i in order:
        c = cases[i]
        if args.mode == "shared":
            O.vlm_shared([c.verts], c.alphas, dtype=np.float32)
        else:
            for a in c.alphas:
                O.vlm_run([c.verts], a, dtype=np.float32)
        done += len(c.alphas)
        used += 1
        if time.perf_counter() - t0 > seconds:
            break
    dt = time.perf_counter() - t0
    sample = "%d of %d cases (%d solves, %d panels max), %.1f s" % (
        used, len(cases), done, max(cases[i].n for i in order[:used]), dt)
    return done / dt, threads, sample


# ---------------------------------------------------------------------------
# clocks during the timed region
# ---------------------------------------------------------------------------
class ClockSampler:
    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index):
        self.index = index
        self.rows = []
        self.proc = None

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.index), "--query-gpu=" + self.Q,
                                          "--format=csv,noheader,nounits", "-lms", "100"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            parts = [x.strip() for x in line.split(",")]
            if len(parts) >= 7:
                self.rows.append(parts)

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        if not self.rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unsampled"]}
        sm = [float(r[0]) for r in self.rows if r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if r[1].replace(".", "").isdigit()]
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        reasons = sorted({names[k] for r in self.rows for k in range(4) if r[3 + k].lower() == "active"})
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "samples": len(self.rows), "reasons": reasons}


# ---------------------------------------------------------------------------
def run_reference(args):
    """The reference arm: the CPU restatement of the reference backend (float,
    all host threads) on the same workload.  One step is a fixed subset of the
    batch: the cases of a stride-7 order (which keeps the subset's size mix
    close to the whole batch's) that the first warm-up pass fits into
    --ref-step-seconds.  --warmup untimed steps, then --steps timed steps of
    exactly that subset; value = solves per step over the mean step time."""
    rank, world, _ = dist_env()
    if rank != 0:
        return
    from oracle import oracle as O
    O.lib()
    threads = O.num_threads()
    cases = workload(args)
    order = stratified_order(cases)

    def solve(c):
        if args.mode == "shared":
            O.vlm_shared([c.verts], c.alphas, dtype=np.float32)
        else:
            for a in c.alphas:
                O.vlm_run([c.verts], a, dtype=np.float32)

    picks, t0 = [], time.perf_counter()
    for i in order:  # first warm-up step: size the subset
        solve(cases[i])
        picks.append(i)
        if time.perf_counter() - t0 > args.ref_step_seconds:
            break
    for _ in range(max(args.warmup, 1) - 1):
        for i in picks:
            solve(cases[i])
    times = []
    for _ in range(args.steps):
        t0 = time.perf_counter()
        for i in picks:
            solve(cases[i])
        times.append(time.perf_counter() - t0)
    step_solves = sum(len(cases[i].alphas) for i in picks)
    ms = 1000.0 * float(np.mean(times))
    rate = step_solves / (ms / 1000.0)
    sample = "%d of %d cases per step (%d solves, %d panels max, size-stratified), %d timed steps" % (
        len(picks), len(cases), step_solves, max(cases[i].n for i in picks), args.steps)
    print(json.dumps({
        "impl": "reference", "metric": METRIC, "value": rate, "unit": "solves/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": max(args.warmup, 1), "ms_per_step": ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": dict(config(args, cases), reference_step=sample),
        "cpu_baseline": {"value": rate, "unit": "solves/s", "cores": threads, "kind": "port", "sample": sample},
        "e2e": {"value": rate, "unit": "solves/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
        "note": "CPU restatement of the reference backend (OpenMP for its Taskflow loops, LAPACK sgetrf/sgetrs "
                "through scipy's OpenBLAS), pinned to the reference's own drivers compiled here; the reference's "
                "ISPC build needs ispc/xmake/Taskflow, absent on this box"}))


def run_gpu(args):
    import torch
    rank, world, local = dist_env()
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl", device_id=dev)
    from tinyvlm_gb300.batch import BatchPipeline, BatchSolver, pack_alphas, pack_verts

    cases = workload(args)
    depth = max(1, args.in_flight)
    # one batch in flight: its own solver, with the plan tuned for one in flight
    bs = BatchSolver(cases, mode=args.mode, refine=args.refine, fp64_residual=args.fp64_residual)
    pipe = BatchPipeline(cases, depth=depth, mode=args.mode, refine=args.refine, fp64_residual=args.fp64_residual,
                         streams=[torch.cuda.Stream(dev) for _ in range(depth)])
    verts_h = torch.from_numpy(pack_verts(cases)).pin_memory()
    alphas = pack_alphas(cases)
    verts_d = verts_h.to(dev)
    stream = torch.cuda.current_stream(dev)
    co_h = torch.zeros((bs.nsolve, 5), dtype=torch.float64).pin_memory().numpy()
    g_h = torch.zeros(bs.gamma_floats, dtype=torch.float32).pin_memory().numpy()

    def barrier():
        if world > 1:
            import torch.distributed as dist
            dist.barrier()

    # warm-up: captures every graph
    torch.cuda.synchronize()
    pipe.set_inputs(verts_d, alphas, ref_pt=(0.25, 0.0, 0.0))
    for _ in range(max(args.warmup, 3) * depth):
        pipe.run()
    bs.set_inputs(verts_d, alphas, ref_pt=(0.25, 0.0, 0.0), stream=stream)
    for _ in range(max(args.warmup, 3)):
        bs.run(stream=stream)
    torch.cuda.synchronize()

    # --- device-resident throughput, one batch in flight ----------------------
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(stream)
    for _ in range(args.steps):
        bs.run(stream=stream)
    e1.record(stream)
    torch.cuda.synchronize()
    barrier()
    ms1 = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)
    value1 = replica_value(bs.nsolve, world, ms1)

    # --- device-resident throughput, `depth` batches in flight ---------------
    # each slot's stream starts after e0; the timed region ends when every
    # slot's last batch has finished
    barrier()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with ClockSampler(local) as clk:
        e0.record(stream)
        for st in pipe.streams:
            st.wait_event(e0)
        for _ in range(args.steps):
            pipe.run()
        for st in pipe.streams:
            stream.wait_stream(st)
        e1.record(stream)
        torch.cuda.synchronize()
    barrier()
    ms = max_over_ranks(e0.elapsed_time(e1) / args.steps, world, dev)
    value = replica_value(bs.nsolve, world, ms)

    # --- end to end through the public API with host buffers ----------------
    # one batch in flight: inputs in, solve, results out, per step
    lat1 = []
    barrier()
    torch.cuda.synchronize()
    for _ in range(args.steps):
        s0 = time.perf_counter()
        bs.set_inputs(verts_h, alphas, ref_pt=(0.25, 0.0, 0.0), stream=stream)
        bs.run(want_gamma=True, stream=stream)
        bs.results_into(co_h, g_h, stream=stream)
        lat1.append(1000.0 * (time.perf_counter() - s0))
    torch.cuda.synchronize()
    # `depth` in flight: batch i+1 is submitted before batch i is collected;
    # a batch's latency runs from its submit to the end of its collect
    lat, t_sub = [], {}
    barrier()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(args.steps):
        if pipe.full():
            t, _, _ = pipe.collect(co_h, g_h)
            lat.append(1000.0 * (time.perf_counter() - t_sub.pop(t)))
        s0 = time.perf_counter()
        t_sub[pipe.submit(verts_h, alphas, ref_pt=(0.25, 0.0, 0.0), want_gamma=True)] = s0
    while pipe.pending():
        t, _, _ = pipe.collect(co_h, g_h)
        lat.append(1000.0 * (time.perf_counter() - t_sub.pop(t)))
    torch.cuda.synchronize()
    e2e_ms = max_over_ranks(1000.0 * (time.perf_counter() - t0) / args.steps, world, dev)
    e2e = replica_value(bs.nsolve, world, e2e_ms)
    h2d = verts_h.numel() * 4 + alphas.nbytes
    d2h = co_h.nbytes + g_h.nbytes

    # --- per-stage CUDA-event profile (same stream) --------------------------
    prof = bs.profile(stream=stream)
    prof2 = bs.profile(stream=stream)
    prof = {k: min(prof[k], prof2[k]) for k in prof}
    co_ref, _ = bs.results(stream=stream)
    plain = plain_path_rate(args, cases, dev, co_ref if args.mode == "exact" else None) if rank == 0 else None
    cpu = None
    if rank == 0 and not args.no_cpu_baseline:
        rate, threads, sample = cpu_sample(args, cases, args.cpu_seconds)
        cpu = {"value": rate, "unit": "solves/s", "cores": threads, "kind": "port", "sample": sample}
    if rank != 0:
        return

    peaks = {}
    pk = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(pk):
        peaks = json.load(open(pk))
    roof = roofline(bs, stream, peaks, ms)
    configs = None
    if not args.no_configs:
        # the other configurations, one short record each (outside the timed region of the headline)
        configs = {}
        for name, fn in (("A_elliptic16x16", lambda: config_a()),
                         ("B_uvlm_20x80_500_steps", lambda: config_b(500)),
                         ("C_elliptic128x128_64_alphas", lambda: config_c(128, 3, args.refine)),
                         ("D_exact_formulation", lambda: exact_mode_rate(cases, 5, args.refine)),
                         ("E_served_mixed_stream", lambda: config_e((16.0,), 30)),
                         ("E_uvlm_step_paths", lambda: uvlm_step_paths(50))):
            t0 = time.perf_counter()
            try:
                with ClockSampler(local) as cclk:
                    configs[name] = fn()
                configs[name]["clocks"] = cclk.summary()
            except Exception as e:  # a failing side workload must not hide the headline
                configs[name] = {"error": "%s: %s" % (type(e).__name__, e)}
            configs[name]["wall_s"] = time.perf_counter() - t0
    out = {
        "metric": METRIC, "value": value, "unit": "solves/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32+f64", "data": "synthetic (seeded trapezoidal wings)",
        "config": dict(config(args, cases), in_flight=depth),
        "e2e": {"value": e2e, "unit": "solves/s", "h2d_bytes_per_step": int(h2d), "d2h_bytes_per_step": int(d2h)},
        "latency_ms": {"p50": float(np.percentile(lat, 50)), "p99": float(np.percentile(lat, 99)),
                       "what": "per batch of %d solves, submit to collected results, %d batches in flight "
                               "(BatchPipeline)" % (bs.nsolve, depth)},
        "one_in_flight": {"value": value1, "ms_per_step": ms1, "unit": "solves/s", "tuning": bs.tuning,
                          "latency_ms": {"p50": float(np.percentile(lat1, 50)), "p99": float(np.percentile(lat1, 99)),
                                         "what": "per batch, set_inputs + run + results through BatchSolver"}},
        "gpu_launches": int(pipe.launches()) * args.steps,  # the pipeline's plan: the headline's timed region
        "clocks": clk.summary(),
        "roofline": roof,
        "stage_ms": prof,
        "plain_fp64_gpu": plain,
        "cpu_baseline": cpu,
        "tuning": pipe.tuning,
        "configs": configs,
    }
    print(json.dumps(out))


# DRAM bytes per algorithmic byte of the tensor-core trailing update
# (dram__bytes_read.sum + dram__bytes_write.sum of k_update_tc over the
# launches' algorithmic bytes; the operands are re-read from L2, not DRAM),
# from one ncu capture of this batch (512 cases, the one-in-flight plan whose
# update the roofline entry times): one step, 31 launches, 4.88 GB of DRAM
# traffic over 7.60 GB algorithmic
TC_TRAFFIC_PER_ALG_BYTE = 0.643


def roofline(bs, stream, peaks, ms_step):
    """Roofline entry of the LU's tensor-core trailing update (k_update_tc),
    the largest kernel of the batched step: algorithmic bytes per launch
    (C read and written, L21 and U12 read once) over its CUDA-event time per
    launch, against the measured HBM copy bandwidth (the update is
    bandwidth-bound: 2W/8 = 32 flop per byte at W = 128)."""
    up = bs.update_profile(stream=stream)
    if up["launches"] == 0 or up["ms"] <= 0:
        return None
    hbm = peaks.get("hbm_gbs")
    src = "MEASURED_PEAKS.json hbm_gbs (of measured)"
    if hbm is None:
        hbm, src = 6800.0, "fallback 6.8 TB/s (of fallback)"
    t = up["ms"] / 1000.0 / up["launches"]
    per_launch = up["bytes"] / up["launches"]
    achieved = per_launch / t / 1e9
    traffic = per_launch * TC_TRAFFIC_PER_ALG_BYTE if TC_TRAFFIC_PER_ALG_BYTE else None
    return {"kernel": "k_update_tc (LU trailing update, tcgen05 kind::tf32, 3xTF32)", "bound": "hbm",
            "achieved": achieved, "peak": hbm, "unit": "GB/s", "frac": achieved / hbm, "traffic": traffic,
            "peak_source": src, "launches": up["launches"], "ms_total": up["ms"],
            "share_of_step": up["ms"] / ms_step,
            "tflops_alg": up["flops"] / (up["ms"] / 1000.0) / 1e12,
            "work": "per outer block and system: 8 m^2 + 8 m W bytes, 2 m^2 W flops (m = n - kend, W = 128)"}


def plain_path_rate(args, cases, dev, co):
    """The plain per-solve GPU path (one VLM::run per solve) on a sample of the
    cases, in double (the comparison the batched path is held to) and in
    float, and the batched path's CL/CM deviation from the double results."""
    if args.plain_solves <= 0:
        return None
    import torch
    from tinyvlm_gb300.vlm import VLM, FlowData
    start = np.cumsum([0] + [len(c.alphas) for c in cases])
    picks, total = [], 0
    for i in range(0, len(cases), 7):
        picks.append(i)
        total += len(cases[i].alphas)
        if total >= args.plain_solves:
            break

    def timed(prec):
        sims = {i: VLM("gb300", [cases[i].verts], precision=prec) for i in picks}
        res = []
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        for i in picks:
            for q, a in enumerate(cases[i].alphas):
                res.append((start[i] + q, sims[i].run(FlowData(a), ref_pt=(0.25, 0.0, 0.0))))
        torch.cuda.synchronize()
        return res, time.perf_counter() - t0

    res, dt = timed(64)
    res32, dt32 = timed(32)
    out = {"value": len(res) / dt, "unit": "solves/s", "solves": len(res),
           "what": "plain per-solve double GPU path (VLM::run semantics, one solve per call, double throughout)",
           "fp32": {"value": len(res32) / dt32, "unit": "solves/s", "solves": len(res32),
                    "what": "the same calls with the float kernels (the reference's float backend semantics)",
                    "max_rel_err_cl_vs_fp64": max(abs(b.cl - a.cl) / max(abs(a.cl), 1e-3)
                                                  for (_, a), (_, b) in zip(res, res32))}}
    if co is not None:  # same formulation (per-alpha AIC) only
        cl_err = max(abs(co[k, 0] - r.cl) / max(abs(r.cl), 1e-3) for k, r in res)
        cm_err = max(float(np.abs(co[k, 2:5] - np.array(r.cm)).max() / max(np.abs(r.cm).max(), 1e-6)) for k, r in res)
        out["batched_vs_plain"] = {"max_rel_err_cl": cl_err, "max_rel_err_cm": cm_err, "target": 1e-5}
    return out


def reference_mesh(name):
    """A mesh of the reference's mesh/ directory, (4, nc+1, ns+1) float32, quarter-chord shifted, from the
    committed fixture tests/golden/ref_meshes.npz (the numbers the reference's own plot3d reader returns)."""
    from tinyvlm_gb300 import mesh as M
    xyz = np.load(os.path.join(ROOT, "tests", "golden", "ref_meshes.npz"))[name]
    v = np.ones((4,) + xyz.shape[1:], np.float32)
    v[:3] = xyz
    M.quarter_chord(v)
    return v


def config_c(n=128, steps=3, refine=1, geometry="reference"):
    """Config C: elliptic n x n wing (16,384 panels at n = 128), 64 alphas in [-10, 10] deg on one AIC.
    geometry "reference": the reference's mesh/elliptic_128x128.x (tip chord 0.0707); "generated": the
    literal analytic planform with a zero tip chord, whose AIC is singular to working precision at this
    spanwise count (its errors measure the conditioning, not the solver).

    Float AIC, tensor-core LU and refinement with the FP64 residual (the
    batched path with GBVLM_BATCH_FP64_RESIDUAL: the residual's AIC is the
    float one plus its float-pair correction), timed with CUDA events; then
    every alpha's error against the full double solve of the same system on
    the device (double assembly, double LU, gbvlm_vlm_run_shared at
    precision 64, which the tests hold to the oracle's LAPACK dgetrf/dgetrs
    at 1e-9): ||gamma - gamma_64|| / ||gamma_64||, and CL and CM_y relative
    errors guarded near zero lift (denominator at least 1e-3 of the sweep's
    largest value).  The same plan without the correction (residual of the
    stored float AIC) is timed and its errors reported beside it."""
    from tinyvlm_gb300 import device as D
    from tinyvlm_gb300 import mesh as M
    from tinyvlm_gb300.batch import BatchSolver, pack_alphas, pack_verts
    from tinyvlm_gb300.vlm import VLM
    if geometry == "reference":
        v = reference_mesh("elliptic_%dx%d" % (n, n))
    else:
        v = M.elliptic(n, n).astype(np.float32)
        M.quarter_chord(v)
    al = np.radians(np.linspace(-10.0, 10.0, 64))
    case = M.Case(v, al, {})

    def measure(fp64_residual):
        bs = BatchSolver([case], mode="shared", refine=refine, fp64_residual=fp64_residual)
        stream = D.Stream()
        bs.set_inputs(pack_verts([case]), pack_alphas([case]), ref_pt=(0.0, 0.0, 0.0), stream=stream)
        bs.run(stream=stream)
        stream.synchronize()
        prof = bs.profile(stream=stream)
        e0, e1 = D.Event(), D.Event()
        e0.record(stream)
        for _ in range(steps):
            bs.run(stream=stream)
        e1.record(stream)
        stream.synchronize()
        ms = e0.elapsed_time(e1) / steps
        bs.run(want_gamma=True, stream=stream)
        co, gam = bs.results(gamma=True, stream=stream)
        out = dict(ms=ms, prof=prof, co=co, gam=gam, lu_flops=bs.lu_flops, interactions=bs.interactions,
                   tuning=bs.tuning, arena_bytes=bs.arena_bytes)
        del bs
        D.synchronize()
        return out

    flt = measure(False)
    m = measure(True)
    t0 = time.perf_counter()
    ref, g64 = VLM("gb300", [v], precision=64).run_shared(al, return_gamma=True)
    t64 = time.perf_counter() - t0
    cl64 = np.array([r.cl for r in ref])
    cm64 = np.array([r.cm[1] for r in ref])
    g_cl, g_cm = 1e-3 * np.abs(cl64).max(), 1e-3 * np.abs(cm64).max()

    def errors(r):
        co, gam = r["co"], r["gam"]
        e_cl = [float(abs(co[k, 0] - cl64[k]) / max(abs(cl64[k]), g_cl)) for k in range(64)]
        e_cm = [float(abs(co[k, 3] - cm64[k]) / max(abs(cm64[k]), g_cm)) for k in range(64)]
        e_g = [float(np.linalg.norm(gam[k].astype(np.float64) - g64[k]) / np.linalg.norm(g64[k])) for k in range(64)]
        return e_cl, e_cm, e_g

    e_cl, e_cm, e_g = errors(m)
    f_cl, f_cm, f_g = errors(flt)
    prof = m["prof"]
    lu = m["lu_flops"] / (prof["lu_factor"] / 1000.0) / 1e12
    asm = FLOP_PER_INTERACTION * m["interactions"] / (flt["prof"]["assembly"] / 1000.0) / 1e12
    ms = m["ms"]
    return {"workload": "large steady: elliptic %dx%d = %d panels (%s geometry), 64 alphas, one AIC" %
                        (n, n, n * n, geometry),
            "ms_per_run": ms, "solves_per_s": 64 / (ms / 1000.0), "stage_ms": prof, "lu_tflops": lu,
            "assembly_tflops_alg": asm,
            "assembly_correction_ms": prof["assembly"] - flt["prof"]["assembly"],
            "refine_iters": refine, "residual": "fp64 (float AIC + float-pair correction)",
            "arena_bytes": m["arena_bytes"], "tuning": m["tuning"],
            "error_vs_fp64": {"alpha_deg": [round(float(a), 4) for a in np.degrees(al)], "cl_rel": e_cl,
                              "cm_rel": e_cm, "gamma_rel_norm": e_g,
                              "max": {"cl": max(e_cl), "cm": max(e_cm), "gamma": max(e_g)}, "target": 1e-5,
                              "reference": "device double assembly + double LU of the same system (plain "
                                           "per-operator path, gbvlm_vlm_run_shared precision 64)"},
            "float_residual": {"what": "the same plan, residual of the stored float AIC",
                               "ms_per_run": flt["ms"], "solves_per_s": 64 / (flt["ms"] / 1000.0),
                               "stage_ms": flt["prof"],
                               "max_error_vs_fp64": {"cl": max(f_cl), "cm": max(f_cm), "gamma": max(f_g)}},
            "plain_fp64_sweep_s": t64, "plain_fp64_solves_per_s": 64 / t64}


def run_large(args):
    print(json.dumps(config_c(args.large_n, args.steps, args.refine, args.large_geometry)))


def config_a(repeats=50):
    """Config A: the elliptic 16 x 16 half wing (b = 10, root chord 1, cosine spanwise spacing), alpha = 5
    deg, one VLM::run per call through the plain per-solve path: float (the reference's semantics) and
    double; latency per solve (median over `repeats` calls, each with its read-back) and CL."""
    from tinyvlm_gb300 import mesh as M
    from tinyvlm_gb300.vlm import VLM, FlowData
    v = M.elliptic(16, 16).astype(np.float32)
    M.quarter_chord(v)
    out = {"workload": "elliptic 16x16 = 256 panels, alpha 5 deg, VLM::run per call"}
    for prec in (32, 64):
        sim = VLM("gb300", [v], precision=prec)
        fl = FlowData(math.radians(5.0))
        sim.run(fl)
        lat = []
        for _ in range(repeats):
            t0 = time.perf_counter()
            r = sim.run(fl)
            lat.append(1000.0 * (time.perf_counter() - t0))
        out["fp%d" % prec] = {"cl": r.cl, "cdi": r.cd, "p50_ms": float(np.percentile(lat, 50)),
                              "p99_ms": float(np.percentile(lat, 99)), "solves_per_s": 1000.0 / float(np.median(lat))}
    out["cl_fp32_vs_fp64"] = abs(out["fp32"]["cl"] - out["fp64"]["cl"]) / abs(out["fp64"]["cl"])
    return out


def pitch_plunge_assembly(k=0.5):
    """Config B's motion: heave 0.1 sin(kt), pitch 3 deg sin(kt + 90 deg) about the quarter chord, u = 1."""
    from tinyvlm_gb300.kinematics import Assembly, KinematicsTree, rotation_matrix, sin, translation_matrix
    tree = KinematicsTree()
    fs = tree.add(lambda t: translation_matrix([-t, 0.0, 0.0]))
    heave = tree.add(lambda t: translation_matrix([0.0, 0.0, 0.1 * sin(k * t)])).after(fs)
    pitch = tree.add(lambda t: rotation_matrix([0.25, 0, 0], [0, 1, 0], math.radians(3.0) * sin(k * t + math.pi / 2))).after(heave)
    asm = Assembly(fs)
    asm.add("wing", pitch)
    return asm


def config_b(steps=500, rollup=False):
    """Config B: 20 x 80 rectangular half wing (chord 1, semispan 4), the pitch-plunge motion, dt = 0.05.
    The float device time loop (reference semantics) timed end to end, and its CL(t) and CM_y(t) against
    the double device time loop of the same run at every step (the double path matches the oracle's
    double time loop to 1e-9 in the tests; the reference's own float CL(t) is pinned there to 2e-5)."""
    from tinyvlm_gb300 import device as D
    from tinyvlm_gb300 import mesh as M
    from tinyvlm_gb300.uvlm import UVLM
    v = M.rectangular(20, 80, 1.0, 4.0).astype(np.float32)
    M.quarter_chord(v)
    asm = pitch_plunge_assembly()
    sim = UVLM("gb300", [v], precision=32)
    sim.run(asm, t_steps=8, dt=0.05)  # warm-up
    D.synchronize()
    t0 = time.perf_counter()
    r32 = sim.run(asm, t_steps=steps, dt=0.05, rollup=rollup)
    D.synchronize()
    s32 = time.perf_counter() - t0
    t0 = time.perf_counter()
    r64 = UVLM("gb300", [v], precision=64).run(asm, t_steps=steps, dt=0.05, rollup=rollup)
    D.synchronize()
    s64 = time.perf_counter() - t0
    rec = slice(1, steps - 1)
    cl_scale = float(np.abs(r64["cl"][rec]).max())
    cm_scale = float(np.abs(r64["cm"][rec, 1]).max())
    e_cl = np.abs(r32["cl"][rec] - r64["cl"][rec]) / cl_scale
    e_cm = np.abs(r32["cm"][rec, 1] - r64["cm"][rec, 1]) / cm_scale
    return {"workload": "UVLM pitch-plunge: rectangular 20x80 = 1600 panels, %d steps, dt 0.05, rollup %d, "
                        "wake %d rings at the end" % (steps, int(rollup), 80 * (steps - 1)),
            "float_s": s32, "steps_per_s": steps / s32, "double_s": s64,
            "tuning": getattr(sim, "tuning", None),
            "error_float_vs_double": {"cl_max_over_max_abs": float(e_cl.max()),
                                      "cm_y_max_over_max_abs": float(e_cm.max()),
                                      "cl_at_step_100_200_300_400_498": [float(e_cl[k - 1]) for k in
                                                                         (100, 200, 300, 400, steps - 2) if
                                                                         k - 1 < e_cl.size]},
            "cl_last": float(r32["cl"][steps - 2])}


def run_uvlm(args):
    """Config B (see config_b), plus the CPU restatement timed on its first 40 steps."""
    out = config_b(args.uvlm_steps, bool(args.rollup))
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        from tinyvlm_gb300 import device as D
        from tinyvlm_gb300 import mesh as M
        from tinyvlm_gb300.uvlm import UVLM, kinematics_arrays
        v = M.rectangular(20, 80, 1.0, 4.0).astype(np.float32)
        M.quarter_chord(v)
        asm = pitch_plunge_assembly()
        steps = 40
        T, Td, fsv, ref = kinematics_arrays(asm, steps, 0.05)
        t0 = time.perf_counter()
        O.uvlm_run([v], [True], T, Td, fsv, ref, steps, 0.05, dtype=np.float32, rollup=False)
        cpu = time.perf_counter() - t0
        sim = UVLM("gb300", [v], precision=32)
        D.synchronize()
        t0 = time.perf_counter()
        sim.run(asm, t_steps=steps, dt=0.05, rollup=False)
        D.synchronize()
        out["cpu_baseline"] = {"sample": "first %d steps" % steps, "cpu_s": cpu, "gpu_s": time.perf_counter() - t0,
                               "cores": O.num_threads(), "kind": "port"}
    print(json.dumps(out))


def run_aero2dof(args):
    """Coupled pitch-plunge UVLM (the reference's tests/uvlm_2dof.cpp run): wing + flap pair (chord 1, span
    40,000, 2 x 2 panels each), the reference's parameters, t_final 1000 (2000 steps of dt 0.5); float
    aerodynamics, double Newmark structure, Newton loop per step on the device.  The CPU leg runs the
    oracle's restatement of the same loop (double) on the first steps."""
    import torch
    from tinyvlm_gb300 import mesh as M
    from tinyvlm_gb300.aeroelastic import UVLM_2DOF, reference_vars
    v = M.rectangular(4, 2, 1.0, 40000.0).astype(np.float32)
    M.quarter_chord(v)
    surfaces = [np.ascontiguousarray(v[:, :3, :]), np.ascontiguousarray(v[:, 2:, :])]
    vars = reference_vars()
    sim = UVLM_2DOF(surfaces, [0, 1])
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    r = sim.run(vars, 1000.0)
    torch.cuda.synchronize()
    gpu = time.perf_counter() - t0
    n = len(r["iters"])
    out = {"workload": "coupled 2-DOF pitch-plunge UVLM, wing + flap 2x2 + 2x2 panels, U_a = 7, %d steps" % n,
           "gpu_s": gpu, "ms_per_step": 1000.0 * gpu / n, "newton_iters_mean": float(np.mean(r["iters"])),
           "pitch_amplitude_last_quarter_rad": float(np.abs(r["u"][-n // 4:, 1]).max()),
           "plunge_amplitude_last_quarter": float(np.abs(r["u"][-n // 4:, 0]).max())}
    if not args.no_cpu_baseline:
        from oracle import oracle as O
        steps = 200
        t0 = time.perf_counter()
        O.aero2dof_run(surfaces, [0, 1], vars, 1000.0, steps=steps)
        out["cpu_ms_per_step_first%d" % steps] = 1000.0 * (time.perf_counter() - t0) / steps
        out["cpu_note"] = "oracle restatement (numpy driver over the C operators), one thread for these sizes"
    print(json.dumps(out))


def run_nlvlm(args):
    """Nonlinear VLM (the reference's tests/nlvlm_curves.cpp case): the 5 x 200 "infinite" rectangle at
    alpha = 19 deg, strip angles corrected toward three tabulated lift curves (100 points, 0-20 deg); float,
    the iteration loop on the device with one error read per iteration.  The CPU leg runs the oracle's
    restatement of the same loop."""
    import math
    import torch
    from tinyvlm_gb300 import mesh as M
    from tinyvlm_gb300.vlm import NLVLM, Database, FlowData, WingProfile

    def spallart(cl0, a0, a1, cla0, cla1):
        return lambda a: cla0 * a + 0.5 * (cl0 - cla1 * a) * (1.0 + math.erf((a - a0) / a1))
    curves = {"spallart1": spallart(1.2, 0.28, 0.02, 2 * math.pi, 2 * math.pi),
              "spallart2": spallart(0.72, 0.28, 0.04, 2 * math.pi, 1.5 * math.pi),
              "polar": lambda a: 2 * math.pi * a}
    v = M.rectangular(5, 200, 1.0, 40000.0).astype(np.float32)
    M.quarter_chord(v)
    alpha = math.radians(19.0)
    db_a = np.linspace(0.0, math.radians(20.0), 100).astype(np.float32)
    sim = NLVLM("gb300", [v])
    out = {"workload": "NLVLM, 5x200 rectangle (1000 panels), alpha 19 deg, three lift curves", "runs": {}}
    for name, f in curves.items():
        db = Database()
        db.profiles.append(WingProfile(db_a, np.array([f(float(a)) for a in db_a], np.float32)))
        sim.run(FlowData(alpha), db)  # warm-up
        torch.cuda.synchronize()
        reps = 20
        t0 = time.perf_counter()
        for _ in range(reps):
            res = sim.run(FlowData(alpha), db)
        torch.cuda.synchronize()
        ms = 1000.0 * (time.perf_counter() - t0) / reps
        row = {"gpu_ms_per_run": ms, "iters": sim.iters, "cl": res.cl, "cl_rel_err_vs_curve": abs(res.cl - f(alpha)) / f(alpha)}
        if not args.no_cpu_baseline:
            from oracle import oracle as O
            t0 = time.perf_counter()
            O.nlvlm_run([v], alpha, db_a, db.profiles[0].CL)
            row["cpu_ms_per_run"] = 1000.0 * (time.perf_counter() - t0)
        out["runs"][name] = row
    out["note"] = "per run: AIC assembly and factorisation, then the iterations; the CPU leg is the oracle (numpy driver over the C operators)"
    print(json.dumps(out))


def run_hbvlm(args):
    """HBVLM 2-DOF residual solves (the served workload's third kind): section wing 45 x 1, 5 harmonics (11 time
    instances, 495 unknowns), Anderson acceleration with history 10 on the device; six seeded requests, each
    solved from rest.  Reports ms per solve and Anderson iterations."""
    import torch
    from tinyvlm_gb300 import serve as S
    make = S.hbvlm_factory()
    hb = make()
    rng = np.random.default_rng(SEED)
    reqs = [S.hbvlm_request(rng) for _ in range(6)]
    ft = np.zeros((2, 11))
    for om, dyn in reqs[:2]:  # warm-up
        hb.gamma_coeffs[:] = 0.0
        hb.run(om, dyn, ft)
    torch.cuda.synchronize()
    ms, its = [], []
    for om, dyn in reqs:
        hb.gamma_coeffs[:] = 0.0
        t0 = time.perf_counter()
        hb.run(om, dyn, ft)
        torch.cuda.synchronize()
        ms.append(1000.0 * (time.perf_counter() - t0))
        its.append(int(hb.iterations))
    # the 3-point finite-difference Jacobian of the loads with respect to the 22 motion coefficients
    # (scripts/finite_diff.py:26-48 as scripts/continuation.py:192-195 uses it): 44 HBVLM solves, as one
    # batch (run_batch) and one run at a time
    from tinyvlm_gb300.finite_diff import numerical_jac_batch, perturbed_points
    om, dyn = reqs[0]
    x = dyn.ravel().copy()
    x[x == 0] = 1e-3

    def f_batch(points):
        fl = [np.zeros((2, 11)) for _ in points]
        hb.gamma_coeffs[:] = 0.0
        hb.run_batch([om] * len(points), [p.reshape(2, -1) for p in points], fl)
        return [f.ravel() for f in fl]

    numerical_jac_batch(f_batch, x)  # warm-up
    jb = []
    for _ in range(3):
        torch.cuda.synchronize()
        t0 = time.perf_counter()
        numerical_jac_batch(f_batch, x)
        torch.cuda.synchronize()
        jb.append(1000.0 * (time.perf_counter() - t0))
    pts, _ = perturbed_points(x)
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for p in pts:
        hb.gamma_coeffs[:] = 0.0
        hb.run(om, p.reshape(2, -1), ft)
    torch.cuda.synchronize()
    seq = 1000.0 * (time.perf_counter() - t0)
    print(json.dumps({"workload": "HBVLM 2-DOF section 45x1, H = 5, Anderson m = 10 on the device, 6 seeded requests",
                      "ms_per_solve": ms, "median_ms": float(np.median(ms)), "anderson_iters": its,
                      "fd_jacobian": {"sets": len(pts), "batched_ms": float(np.median(jb)),
                                      "one_run_per_set_ms": seq}}))


def config_e(rates=(2.0, 8.0, 32.0), requests=45, seed=SEED):
    """Config E: Poisson mixed stream in equal thirds -- steady VLM on trapezoids of 256-16,384 panels
    (log-uniform), single UVLM steps on a resident 20x80 wing with a 500-row (40,000-ring) wake, 2-DOF
    HBVLM residuals (45 x 1 section, 5 harmonics = 11 instances) -- through the server's lanes; per
    arrival rate: p50/p99 latency (arrival to result), throughput, steady solves/s."""
    from tinyvlm_gb300 import serve as S
    rng = np.random.default_rng(seed)
    total = len(rates) * requests
    uvlm = S.resident_uvlm(warm_steps=500, capacity=total + 8)
    srv = S.Server(lanes=3, hbm_budget=48 << 30, max_batch=64, uvlm=uvlm, hbvlm=S.hbvlm_factory(45, 5)).start()
    out = {"workload": "served mixed stream (steady 256-16384 panels / UVLM step on a 40,000-ring wake / "
                       "HBVLM 2-DOF 45x1, H=5), Poisson arrivals", "lanes": 3, "budget_bytes": srv.budget,
           "rates": []}
    rid = 0
    for lam in rates:
        reqs = []
        t = time.perf_counter()
        for _ in range(requests):
            t += rng.exponential(1.0 / lam)
            kind = ("steady", "uvlm", "hbvlm")[int(rng.integers(0, 3))]
            payload = (S.steady_case(rng),) if kind == "steady" else (S.hbvlm_request(rng) if kind == "hbvlm" else None)
            reqs.append((t, kind, payload))
        done = []
        for (ta, kind, payload) in reqs:
            now = time.perf_counter()
            if ta > now:
                time.sleep(ta - now)
            done.append(srv.submit(S.Request(rid, kind, payload, arrival=ta)))
            rid += 1
        for r in done:
            r.done.wait(srv.wait_s)
        fin = [r for r in done if r.finish is not None]
        lat = np.array([r.latency for r in fin]) * 1000.0
        span = max(r.finish for r in fin) - min(r.arrival for r in done)
        steady = sum(len(r.payload[0].alphas) for r in fin if r.kind == "steady" and r.error is None)
        row = {"rate_req_s": lam, "completed": len(fin), "errors": sum(r.error is not None for r in done),
               "throughput_req_s": len(fin) / span, "steady_solves_per_s": steady / span,
               "p50_ms": float(np.percentile(lat, 50)), "p99_ms": float(np.percentile(lat, 99))}
        for kind in ("steady", "uvlm", "hbvlm"):
            lk = np.array([r.latency for r in fin if r.kind == kind]) * 1000.0
            if lk.size:
                row[kind] = {"n": int(lk.size), "p50_ms": float(np.percentile(lk, 50)),
                             "p99_ms": float(np.percentile(lk, 99))}
        out["rates"].append(row)
    srv.shutdown()
    out["stats"] = dict(srv.stats)
    return out


def uvlm_step_paths(n=50):
    """One served UVLM step on the resident 20 x 80 wing with a 500-row (40,000-ring) wake, three ways:
    host-launched operators (gbvlm_uvlm_step), one graph launch (gbvlm_uvlm_step_graph) and the
    device-resident request loop (gbvlm_uvlm_loop_*), each with its coefficients read back; per-step
    latency p50/p99 over n steps each, and the loop's throughput with n requests in flight."""
    import ctypes
    from tinyvlm_gb300 import serve as S
    from tinyvlm_gb300._lib import P, call
    sim = S.resident_uvlm(warm_steps=500, capacity=5 * n + 8)
    i, cl, cm = ctypes.c_int64(), ctypes.c_double(), (ctypes.c_double * 3)()

    def lat(fn):
        out = []
        for _ in range(n):
            t0 = time.perf_counter()
            fn()
            out.append((time.perf_counter() - t0) * 1000.0)
        return {"p50_ms": float(np.percentile(out, 50)), "p99_ms": float(np.percentile(out, 99))}

    res = {"workload": "UVLM step on the resident 20x80 wing, wake of 500+ rows (40,000+ rings)"}
    res["host_launched"] = lat(lambda: call("gbvlm_uvlm_step", sim.h, ctypes.cast(ctypes.pointer(i), P),
                                            ctypes.cast(ctypes.pointer(cl), P), ctypes.cast(cm, P), None))
    res["graph"] = lat(lambda: call("gbvlm_uvlm_step_graph", sim.h, ctypes.cast(ctypes.pointer(i), P),
                                    ctypes.cast(ctypes.pointer(cl), P), ctypes.cast(cm, P), None))
    loop = S.UvlmLoop(sim, 0.05)
    try:
        res["device_loop"] = lat(lambda: loop.wait(loop.submit(), 60.0))
        t0 = time.perf_counter()
        tickets = [loop.submit() for _ in range(n)]
        for t in tickets:
            loop.wait(t, 60.0)
        dt = time.perf_counter() - t0
        res["device_loop_pipelined"] = {"steps": n, "steps_per_s": n / dt}
        res["device_loop_stats"] = loop.stats()
    finally:
        loop.close()
    return res


def run_served(args):
    from tinyvlm_gb300 import device as D
    with ClockSampler(int(os.environ.get("LOCAL_RANK", "0"))) as clk:
        out = config_e([float(x) for x in args.rates.split(",")], args.requests)
        out["uvlm_step_paths"] = uvlm_step_paths(50)
        D.synchronize()
    out["clocks"] = clk.summary()
    print(json.dumps(out))


def exact_mode_rate(cases, steps=5, refine=1):
    """The headline batch in the exact formulation (one AIC per case and alpha, the reference's
    alpha-dependent system, VLM::run semantics): solves/s of graph replays, CUDA events."""
    from tinyvlm_gb300 import device as D
    from tinyvlm_gb300.batch import BatchSolver, pack_alphas, pack_verts
    bs = BatchSolver(cases, mode="exact", refine=refine)
    stream = D.Stream()
    bs.set_inputs(D.DeviceArray.from_numpy(pack_verts(cases)), pack_alphas(cases), ref_pt=(0.25, 0.0, 0.0),
                  stream=stream)
    for _ in range(3):
        bs.run(stream=stream)
    e0, e1 = D.Event(), D.Event()
    e0.record(stream)
    for _ in range(steps):
        bs.run(stream=stream)
    e1.record(stream)
    stream.synchronize()
    ms = e0.elapsed_time(e1) / steps
    return {"workload": "the headline batch, exact formulation (%d systems)" % bs.nsys, "ms_per_step": ms,
            "solves_per_s": bs.nsolve / (ms / 1000.0), "tuning": bs.tuning}


def main():
    args = parse()
    if args.impl == "reference":
        run_reference(args)
    elif args.workload == "large":
        run_large(args)
    elif args.workload == "uvlm":
        run_uvlm(args)
    elif args.workload == "aero2dof":
        run_aero2dof(args)
    elif args.workload == "nlvlm":
        run_nlvlm(args)
    elif args.workload == "hbvlm":
        run_hbvlm(args)
    elif args.workload == "served":
        run_served(args)
    else:
        run_gpu(args)


if __name__ == "__main__":
    main()
