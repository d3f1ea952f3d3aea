"""Benchmark: circuit time of the 14-qubit mixed-gate workload (FP64 rho, 4^14
entries = 4.3 GB, 2000 gates drawn uniformly from the 29-entry table on random
distinct qubits), fused passes vs the plain gate-by-gate path, on one GB300.

One step = one run of the whole circuit on the device-resident rho (a CUDA
graph replay of every pass).  ``value`` is seconds per circuit of the fused
path (lower is better), device-timed with CUDA events on the engine's stream.
Extra keys: the plain path's time and the speed-up, the fused-vs-plain error
(the plain path checks every fused result), the roofline of the dominant pass
kernel, ``e2e`` through the C ABI with host buffers (the circuit and rho cross
the host boundary every step), and a CPU baseline of the reference's CPU
algorithm (the oracle port, all host cores) on a bounded systematic sample of
the circuit at full size, with the fused result checked against the
statevector oracle in that CPU leg.

    python bench.py [--gpus 1] [--steps K] [--warmup W] [--impl reference]
                    [--n 14] [--gates 2000] [--planner greedy|learned] [--max-k 4]
"""
import argparse
import json
import os
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path[:0] = [os.path.join(ROOT, "dm-sim_gb300", "python"), ROOT]

import numpy as np  # noqa: E402

import dmsim_workloads as W  # noqa: E402

# DRAM traffic of the pass kernels relative to their algorithmic bytes, from
# ncu captures of two launches each at 12 qubits (dram__bytes_read.sum +
# dram__bytes_write.sum; profiles/k_pass_df64_K4_SPARSE_table_mix_12q.md and
# profiles/k_pass_tc_K4_table_mix_12q.md): reads 268.6 MB of a 268.4 MB state,
# writes equal to the stored runs.  Traffic grows with the state, so a launch's
# traffic is its algorithmic bytes times this ratio.
TRAFFIC_RATIO = 1.0003
TRAFFIC_SOURCE = "ncu DRAM bytes of 2 launches at 12q = 1.0003 x algorithmic, scaled"
CLASS_NAMES = {0: "MOVE", 1: "SIGNED", 2: "PHASE", 3: "DENSE", 4: "SPARSE", 5: "RLIN", 6: "SUPER", 16: "CONVERT",
               17: "TRANSPOSE", 18: "RENORM"}


def peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return d.get("hbm_gbs", 6800.0), "measured"
    return 6800.0, "fallback"


class ClockSampler:
    """nvidia-smi clock/throttle samples every 200 ms during the timed region."""

    FIELDS = "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown," \
             "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown," \
             "clocks_event_reasons.sw_power_cap"

    def __init__(self):
        self.proc = None
        self.lines = []

    def start(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "--query-gpu=" + self.FIELDS, "--format=csv,noheader,nounits",
                                          "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except OSError:
            self.proc = None

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            f = [x.strip() for x in ln.split(",")]
            if len(f) < 9 or f[0] != "0":
                continue
            try:
                sm.append(float(f[1]))
                smax.append(float(f[2]))
            except ValueError:
                continue
            for nm, v in zip(names, f[5:9]):
                if v.lower() == "active":
                    reasons.add(nm)
        return {"sm_mhz": float(np.median(sm)) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


def max_over_ranks(value, world, device):
    """The largest of the ranks' values (the slowest replica's step time):
    an all-reduce MAX over the default process group when world > 1."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist
    t = torch.tensor([value], device=device, dtype=torch.float64)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_seconds_per_circuit(step_ms, world):
    """Whole-job aggregate of the replicas: every rank runs one circuit per
    step, so the job finishes world circuits per (slowest) step time."""
    return step_ms / 1e3 / world


def workload(n, gates):
    return W.table_mix(n, gates, seed=2)


METRIC = "14/16q circuit time, learned-fused vs plain on 1 GB300 at <=1e-10 err; HBM %"


def cpu_stratified(n, circ, stride, offset, threads, fixed_s):
    """Time the reference's CPU algorithm (the oracle port of
    src/dmsim_cpu_omp.hpp) at full size on the systematic sample
    circ[offset::stride] -- every stride-th table gate, so the sample has the
    circuit's mix of basic gates -- and extrapolate to the whole circuit:
    fixed_s (state set-up and the adjoint stage, timed on an empty circuit)
    plus the sample's time per basic gate times the circuit's basic gates.
    Returns (seconds per circuit, seconds the sample took, description)."""
    import oracle as O
    total_basic = sum(O.basic_count(g) for g in circ)
    pre = circ[offset::stride]
    nb = sum(O.basic_count(g) for g in pre)
    t0 = time.perf_counter()
    O.dm_sim(n, pre, nthreads=threads)
    t = time.perf_counter() - t0
    per_basic = max(t - fixed_s, 0.0) / max(nb, 1)
    return fixed_s + per_basic * total_basic, t, \
        f"every {stride}th gate from gate {offset} ({len(pre)} of {len(circ)} gates, {nb} of {total_basic} basic " \
        f"gates) at n={n}, {t:.1f} s, plus {fixed_s:.1f} s fixed (empty circuit), extrapolated per basic gate"


def cpu_fixed_cost(n, threads):
    """Seconds of the reference CPU algorithm's per-run work that does not
    depend on the gates: the state set-up and the adjoint (transpose) stage."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import oracle as O
    O.build()
    t0 = time.perf_counter()
    O.dm_sim(n, [], nthreads=threads)
    return time.perf_counter() - t0


def cpu_stride(n, circ, budget_s):
    """Sampling stride so that one sample takes about budget_s at n qubits
    (measured rate of the oracle port: ~27 ms per basic gate at 14 qubits on
    16 Arm cores, scaling with 4^n)."""
    per_basic = 0.027 * 4.0 ** (n - 14) * 16.0 / max(os.cpu_count() or 1, 1)
    import oracle as O
    total_basic = sum(O.basic_count(g) for g in circ)
    want = max(1.0, budget_s / per_basic)
    return max(1, int(round(total_basic / want)))


def run_reference_arm(args, n, circ):
    """The reference's own CPU algorithm for this path on the machine's host cores:
    each step times one bounded systematic sample of the circuit at full size
    (a different offset per step, so the steps together cover much of it) and
    extrapolates to the whole circuit.  value = mean extrapolated seconds per
    circuit; ms_per_step = the measured time of one step's sample."""
    threads = os.cpu_count() or 1
    fixed = cpu_fixed_cost(n, threads)
    stride = cpu_stride(n, circ, args.cpu_budget)
    for w in range(args.warmup):
        cpu_stratified(n, circ[: 2 * stride], stride, 0, threads, fixed)  # small: page in and spin up threads
    vals, times, samples = [], [], []
    for k in range(args.steps):
        v, t, sample = cpu_stratified(n, circ, stride, (k * 7) % stride, threads, fixed)
        vals.append(v)
        times.append(t)
        samples.append(sample)
    v = float(np.mean(vals))
    line = {"impl": "reference", "metric": METRIC, "value": v,
            "unit": "s/circuit", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": float(np.mean(times)) * 1e3, "higher_is_better": False, "scaling": "weak",
            "vs_baseline": None, "dtype": "f64", "data": "synthetic (seeded circuits, state from |0..0><0..0|)",
            "config": {"workload": f"{n}-qubit mixed-gate circuit: table_mix n={n} gates={len(circ)} seed=2 "
                                   f"(29-entry table, random distinct qubits)", "l2": "inputs larger than L2",
                       "step": "one systematic sample of the circuit at full size, extrapolated per basic gate; "
                               "ms_per_step is the sample's measured time"},
            "value_spread": [float(np.min(vals)), float(np.max(vals))],
            "cpu_baseline": {"value": v, "unit": "s/circuit", "cores": threads, "kind": "port",
                             "cpu": cpu_model(), "sample": samples[0] + f" (step 1 of {args.steps}; offsets vary)"},
            "e2e": {"value": v, "unit": "s/circuit", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line))


def oracle_parity(n, circ, sim):
    """The fused result against the statevector oracle (rho = psi psi^+ for
    these noise-free circuits from a pure state), on the device: fidelity,
    sqrt(1 - F) (an upper bound of the trace distance), max element and
    Frobenius errors.  Part of the CPU leg: the oracle is the checker here."""
    import oracle as O
    sr, si = O.sv_sim(n, circ)
    sim.reset_dm()
    sim.run()
    m = sim.pure_metrics(sr + 1j * si)
    m["sqrt_1_minus_F"] = float(np.sqrt(max(0.0, 1.0 - m["fidelity"])))
    return m


def cpu_model():
    try:
        with open("/proc/cpuinfo") as f:
            txt = f.read()
        for key in ("model name", "CPU part", "Hardware"):
            for ln in txt.splitlines():
                if ln.startswith(key):
                    return f"{key}: {ln.split(':', 1)[1].strip()} ({os.cpu_count()} cores, {os.uname().machine})"
    except OSError:
        pass
    return f"{os.uname().machine}, {os.cpu_count()} cores"


def class_profile(sim, arith_name):
    """One recorded (untimed-by-the-bench) run: per (K, class) launches, device
    ms, share and HBM GB/s from the engine's per-pass CUDA events."""
    import dmsim_gb300 as E
    sim.set_option(E.OPT_RECORD, 1)
    sim.run()
    rec = sim.pass_records()
    run_ms = sim.last_timings()["ms"]
    sim.set_option(E.OPT_RECORD, 0)
    groups = {}
    for r in rec:
        g = groups.setdefault((int(r[0]), int(r[1]), int(r[8])), [0, 0.0, 0.0])
        g[0] += 1
        g[1] += r[6]
        g[2] += r[7]
    tot = sum(g[1] for g in groups.values()) or 1.0
    kernels = {f"K{k}_{CLASS_NAMES[c]}{'_TC' if tc else ''}": {
        "launches": v[0], "ms": round(v[1], 3), "share": round(v[1] / tot, 4),
        "GBps": round(v[2] / max(v[1], 1e-9) / 1e6, 1)} for (k, c, tc), v in sorted(groups.items(), key=lambda kv: -kv[1][1])}
    (dK, dcls, dtc), (dcount, dms, dbytes) = max(groups.items(), key=lambda kv: kv[1][1])
    name = f"k_pass_tc<{dK}> ({CLASS_NAMES[dcls]} operator)" if dtc else f"k_pass<{arith_name},{dK},{CLASS_NAMES[dcls]}>"
    dom = {"kernel": name, "launches": dcount, "ms": dms, "bytes": dbytes, "tc": bool(dtc)}
    return kernels, dom, run_ms


def timed_runs(sim, warmup, steps):
    for _ in range(warmup):
        sim.run()
    ms = []
    for _ in range(steps):
        sim.run()
        ms.append(sim.last_timings()["ms"])
    return float(np.mean(ms))


def extra_workload(args):
    """Measurements beside the bench line (same device timing rules)."""
    import dmsim_gb300 as E
    out = {"workload": args.workload, "steps": args.steps, "warmup": args.warmup}
    clocks = ClockSampler()
    if args.workload == "sweep":
        # 512 hardware-efficient-ansatz circuits, qubits uniform in {6..12},
        # 4-10 layers; one graph-captured launch (work-queue kernel for the
        # narrow circuits, the engine's own kernels for the wide ones) vs
        # sequential plain runs (the reference's method, one circuit at a time)
        ncirc = args.sweep_circuits
        sweep = W.hea_sweep(ncirc, seed=4, nmax=args.sweep_nmax)
        out["sweep"] = {"circuits": ncirc, "qubits": [6, args.sweep_nmax]}
        b = E.Batch([n for n, _ in sweep], mode="fused", max_k=args.max_k)
        for c, (n, circ) in enumerate(sweep):
            b.extend(c, circ)
        b.upload()
        if not args.no_autotune:
            out["autotune_best_ms"] = b.autotune()
        for _ in range(args.warmup):
            b.run()
        clocks.start()
        ms = []
        for _ in range(args.steps):
            b.run()
            ms.append(b.stats()["ms"])
        out["clocks"] = clocks.stop()
        st = b.stats()
        out["batched_s"] = float(np.mean(ms)) / 1e3
        out["batched_circuits_per_s"] = ncirc / out["batched_s"]
        out["batch_stats"] = st
        out["batched_GBps"] = st["bytes"] / (out["batched_s"]) / 1e9
        seq_arms = () if args.no_plain else (("sequential_plain_fp64", dict(mode="plain", plain_arith="fp64")),
                                             ("sequential_plain_df64", dict(mode="plain", plain_arith="df64")),
                                             ("sequential_fused_fp64", dict(mode="fused", fused_arith="fp64")))
        for label, kw in seq_arms:
            seq = 0.0
            worst = 0.0
            for c, (n, circ) in enumerate(sweep):
                with E.Simulation(n, **kw) as s:
                    s.extend(circ)
                    s.upload()
                    s.run()
                    s.run()  # second replay: no first-launch effects
                    seq += s.last_timings()["ms"]
                    if c % 37 == 0:
                        s.reset_dm()
                        s.run()
                        worst = max(worst, float(np.abs(s.get_diag() - b.diag(c)).max()))
            out[label + "_s"] = seq / 1e3
            out[label + "_diag_max_abs_err_vs_batched"] = worst
            out["speedup_batched_vs_" + label] = out[label + "_s"] / out["batched_s"]
        b.close()
    elif args.workload == "peaks":
        # execution-unit throughputs behind the kernels' choice of arithmetic
        rates = E.probe_rates()
        sms = 152
        clk = 2.07e9
        out["ops_per_s"] = rates
        out["per_sm_per_clock_at_2070MHz"] = {k: round(v / sms / clk, 2) for k, v in rates.items()}
        out["fp64_fma_over_fp32_fma"] = rates["fp64_fma"] / rates["fp32_fma"]
        out["int_lop3_over_fp32_fma"] = rates["int_lop3"] / rates["fp32_fma"]
    elif args.workload == "qft16":
        n = 16
        circ = W.qft_then_layers(n, 1000, seed=3)
        tensor = "all" if args.tensor == "all" else int(args.tensor)
        fused = E.Simulation(n, mode="fused", max_k=args.max_k, planner=args.planner, tensor=tensor)
        fused.extend(circ)
        fused.upload()
        clocks.start()
        out["fused_s"] = timed_runs(fused, args.warmup, args.steps) / 1e3
        out["clocks"] = clocks.stop()
        out["fused_passes"], out["basic_gates"] = fused.plan_stats()
        out["fused_GBps"] = fused.last_timings()["bytes"] / out["fused_s"] / 1e9
        fused.reset_dm()
        out["fused_kernels"], _, _ = class_profile(fused, "df64")
        if not args.no_plain:
            plain = E.Simulation(n, mode="plain")
            plain.extend(circ)
            plain.upload()
            out["plain_kernels"], _, pms = class_profile(plain, "df64")
            out["plain_s"] = pms / 1e3
            out["plain_GBps"] = plain.last_timings()["bytes"] / out["plain_s"] / 1e9
            out["speedup_fused_vs_plain"] = out["plain_s"] / out["fused_s"]
            out["fused_vs_plain_error"] = fused.compare(plain)
            plain.close()
        fused.close()
    elif args.workload == "c64_17":
        n = args.c64_n
        circ = W.u3_cx_ccx(n, 1000, seed=5)
        tensor = "all" if args.tensor == "all" else int(args.tensor)
        s = E.Simulation(n, mode="fused", max_k=args.max_k, precision="c64", planner=args.planner, tensor=tensor)
        s.extend(circ)
        s.upload()
        clocks.start()
        out["c64_s"] = timed_runs(s, args.warmup, args.steps) / 1e3
        out["clocks"] = clocks.stop()
        out["passes"], out["basic_gates"] = s.plan_stats()
        out["c64_GBps"] = s.last_timings()["bytes"] / out["c64_s"] / 1e9
        s.reset_dm()
        out["c64_kernels"], _, _ = class_profile(s, "float")
        d = s.get_diag()
        out["trace_fp64_sum"] = float(d.sum())
        s.close()
        # the same circuit truncated to its first 16 qubits: complex64 against FP64
        nt = min(n, 16)
        trunc = [g for g in circ if max(g[1]) < nt]
        a = E.Simulation(nt, mode="fused", max_k=args.max_k, precision="c64")
        a.extend(trunc)
        a.upload()
        a.run()
        bsim = E.Simulation(nt, mode="fused", max_k=args.max_k)
        bsim.extend(trunc)
        bsim.upload()
        bsim.run()
        out["c64_vs_fp64_16q"] = a.compare(bsim)
        a.close()
        bsim.close()
    print(json.dumps(out))


def main():
    # replicas under torchrun: one GPU per rank.  The engine links its own CUDA
    # runtime, so the rank's device is chosen before any CUDA call, for both it
    # and torch, by restricting the visible devices.
    if int(os.environ.get("WORLD_SIZE", "1")) > 1 and "LOCAL_RANK" in os.environ:
        os.environ["CUDA_VISIBLE_DEVICES"] = os.environ["LOCAL_RANK"]
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="engine")
    ap.add_argument("--n", type=int, default=14)
    ap.add_argument("--gates", type=int, default=2000)
    ap.add_argument("--planner", default="greedy")
    ap.add_argument("--max-k", type=int, default=4)
    ap.add_argument("--tensor", default="1", help="tensor-core passes: 0 off, 1 planner's choice, all")
    ap.add_argument("--cpu-budget", type=float, default=None,
                    help="seconds per CPU sample [20 for the cpu_baseline leg, 8 per step of --impl reference]")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-plain", action="store_true")
    ap.add_argument("--e2e-steps", type=int, default=1)
    ap.add_argument("--no-16q", action="store_true", help="skip the 16-qubit configuration")
    ap.add_argument("--sweep-circuits", type=int, default=512, help="sweep workload: number of circuits")
    ap.add_argument("--sweep-nmax", type=int, default=12, help="sweep workload: qubits uniform in {6..nmax}")
    ap.add_argument("--no-autotune", action="store_true", help="sweep workload: the batch's default settings")
    ap.add_argument("--c64-n", type=int, default=17, help="c64_17 workload: qubits")
    ap.add_argument("--workload", default="table14",
                    help="table14 (the bench line), or extra measurements: sweep, qft16, c64_17, peaks")
    args = ap.parse_args()
    if args.workload != "table14":
        return extra_workload(args)

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    n = args.n
    circ = workload(n, args.gates)

    if args.cpu_budget is None:
        args.cpu_budget = 8.0 if args.impl == "reference" else 20.0
    if args.impl == "reference":
        if rank == 0:
            run_reference_arm(args, n, circ)
        return

    import dmsim_gb300 as E  # fails loudly if the engine library is missing

    if world > 1:
        # replicas only: every rank runs the same single-GPU workload on its own device
        import torch
        torch.cuda.set_device(0)  # the only visible device of this rank
        import torch.distributed as dist
        dist.init_process_group("nccl")

    hbm_peak, peak_kind = peaks()
    tensor = "all" if args.tensor == "all" else int(args.tensor)

    # ---- fused path, FP64 width (the headline): the timed steps
    fused = E.Simulation(n, mode="fused", max_k=args.max_k, planner=args.planner, tensor=tensor, fused_arith="fp64")
    t_up0 = time.perf_counter()
    fused.extend(circ)
    fused.upload()
    upload_s = time.perf_counter() - t_up0
    npasses, nbasic = fused.plan_stats()
    upload_bytes = fused.upload_bytes()
    for _ in range(args.warmup):
        fused.run()
    if world > 1:
        dist.barrier()
    clocks = ClockSampler()
    clocks.start()
    t_wall0 = time.perf_counter()
    ms = []
    for _ in range(args.steps):
        fused.run()
        ms.append(fused.last_timings()["ms"])
    wall = time.perf_counter() - t_wall0
    clk = clocks.stop()
    step_ms = max_over_ranks(float(np.mean(ms)), world, "cuda")
    bytes_per_run = fused.last_timings()["bytes"]
    launches_per_run = int(fused.last_timings()["passes"])

    # ---- per-pass profile of one fused run (untimed): the dominant kernel
    kernels, dom, _ = class_profile(fused, "double")
    dom_name, dcount = dom["kernel"], dom["launches"]
    if dom["tc"]:
        dom_name = dom_name.replace("k_pass_tc<", "k_pass_tc64<")
    achieved = dom["bytes"] / (dom["ms"] * 1e-3) / 1e9

    extra = {}
    err = None
    plain_s = plain_bytes = plain_passes = plain_kernels = None
    if not args.no_plain:
        # the other planner on the same circuit
        other = "greedy" if args.planner == "learned" else "learned"
        g = E.Simulation(n, mode="fused", max_k=args.max_k, planner=other, tensor=tensor, fused_arith="fp64")
        g.extend(circ)
        g.upload()
        extra[f"{other}_s"] = timed_runs(g, 1, 2) / 1e3
        extra[f"{other}_passes"] = g.plan_stats()[0]
        g.close()
        # plain path (the reference's method, FP64 arithmetic) and the fused-vs-plain error
        plain = E.Simulation(n, mode="plain", plain_arith="fp64")
        plain.extend(circ)
        plain.upload()
        plain_kernels, _, plain_ms = class_profile(plain, "double")  # per-pass events cost ~us per pass
        plain_s = plain_ms / 1e3
        plain_bytes = plain.last_timings()["bytes"]
        plain_passes = plain.plan_stats()[0]
        fused.reset_dm()
        fused.run()
        err = fused.compare(plain)
        # the double-float variants (48-bit significands, not FP64 width)
        pdf = E.Simulation(n, mode="plain", plain_arith="df64")
        pdf.extend(circ)
        pdf.upload()
        extra["plain_df64_kernels"], _, pdf_ms = class_profile(pdf, "df64")
        extra["plain_df64_s"] = pdf_ms / 1e3
        extra["hbm_GBps_plain_df64_run"] = pdf.last_timings()["bytes"] / (pdf_ms * 1e-3) / 1e9
        extra["plain_df64_vs_plain_error"] = plain.compare(pdf)
        pdf.close()
        fdf = E.Simulation(n, mode="fused", max_k=args.max_k, planner="learned", tensor=tensor, fused_arith="df64")
        fdf.extend(circ)
        fdf.upload()
        extra["fused_df64_s"] = timed_runs(fdf, 2, 2) / 1e3
        extra["fused_df64_kernels"], _, _ = class_profile(fdf, "df64")
        fdf.reset_dm()
        fdf.run()
        extra["fused_df64_vs_plain_error"] = fdf.compare(plain)
        fdf.close()
        plain.close()

    # ---- end to end through the C ABI with host buffers
    N = 1 << (2 * n)
    pre = E.PinnedBuffer(N)
    pim = E.PinnedBuffer(N)
    e2e = []
    for _ in range(args.e2e_steps):
        t0 = time.perf_counter()
        fused.reset()                 # clear the circuit, rho = |0..0><0..0|
        fused.extend(circ)            # the circuit crosses the host boundary
        fused.upload()                # descriptors H2D
        fused.run()
        fused.get_dm_into(pre.array, pim.array)  # rho D2H (the reference's sim() copies it back)
        e2e.append(time.perf_counter() - t0)
    pre.close()
    pim.close()

    cpu = None
    parity = None
    if rank == 0 and not args.no_cpu:
        threads = os.cpu_count() or 1
        fixed = cpu_fixed_cost(n, threads)
        v, _, sample = cpu_stratified(n, circ, cpu_stride(n, circ, args.cpu_budget), 0, threads, fixed)
        cpu = {"value": v, "unit": "s/circuit", "cores": threads, "kind": "port", "cpu": cpu_model(),
               "sample": sample}
        parity = oracle_parity(n, circ, fused)
    fused.close()

    # ---- the 16-qubit FP64 configuration: QFT ladder on an X-Bernoulli input,
    # then 1000 U3/CX layer gates (68.7 GB of state)
    q16 = None
    if rank == 0 and not args.no_16q:
        q16 = config16(args, tensor, not args.no_plain, not args.no_cpu)

    if rank == 0:
        value = whole_job_seconds_per_circuit(step_ms, world)
        line = {
            "metric": METRIC,
            "value": value, "unit": "s/circuit", "n_gpus": args.gpus, "steps": args.steps, "warmup": args.warmup,
            "ms_per_step": step_ms, "higher_is_better": False, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded circuits, state from |0..0><0..0|)",
            "config": {"workload": f"{n}-qubit mixed-gate circuit: table_mix n={n} gates={len(circ)} seed=2 (29-entry table, random distinct qubits)",
                       "planner": args.planner, "max_k": args.max_k, "tensor": args.tensor, "passes": npasses,
                       "basic_gates": nbasic,
                       "l2": "inputs larger than L2 (rho = %.1f GB)" % (16.0 * N / 1e9), "parallelism": "replicas"},
            "state": "FP64 rho in and out; fused passes at FP64 width: 3/4-qubit operators on the tensor cores "
                     "with 7 BF16 digits per operand, exact integer order sums and one rounding to FP64 per output "
                     "(55-bit significands per column), other passes in FP64; plain = the reference's method in FP64",
            "plain_s": plain_s, "plain_passes": plain_passes, "plain_kernels": plain_kernels,
            "speedup_fused_vs_plain": (plain_s / value) if plain_s else None,
            "fused_vs_plain_error": err,
            "hbm_GBps_fused_run": bytes_per_run / (step_ms * 1e-3) / 1e9,
            "hbm_GBps_plain_run": (plain_bytes / plain_s / 1e9) if plain_s else None,
            **extra,
            "roofline": {"bound": "hbm", "kernel": dom_name, "achieved": round(achieved, 1), "peak": hbm_peak,
                         "unit": "GB/s", "frac": round(achieved / hbm_peak, 4),
                         "traffic": round(dom["bytes"] / dcount * TRAFFIC_RATIO),
                         "traffic_source": TRAFFIC_SOURCE, "peak_kind": peak_kind, "launches": dcount},
            "kernels": kernels,
            "e2e": {"value": float(np.mean(e2e)), "unit": "s/circuit",
                    "h2d_bytes_per_step": int(upload_bytes), "d2h_bytes_per_step": int(16 * N)},
            "gpu_launches": launches_per_run * args.steps,
            "clocks": clk,
            "upload_s": upload_s,
            "wall_s_timed": wall,
            "cpu_baseline": cpu,
            "parity_vs_statevector_oracle": parity,
            "config_16q": q16,
        }
        print(json.dumps(line))
    if world > 1:
        dist.destroy_process_group()


def config16(args, tensor, with_plain, with_oracle):
    """The 16-qubit FP64 configuration beside the bench line: learned-fused
    (FP64 width) time, the plain FP64 path's time, their difference and, in
    the CPU leg, the fused result against the statevector oracle."""
    import dmsim_gb300 as E
    n = 16
    circ = W.qft_then_layers(n, 1000, seed=3)
    out = {"workload": "16-qubit QFT ladder on an X-Bernoulli(0.5) input + 1000 U3/CX layer gates, seed 3"}
    f = E.Simulation(n, mode="fused", max_k=args.max_k, planner=args.planner, tensor=tensor, fused_arith="fp64")
    f.extend(circ)
    f.upload()
    out["fused_s"] = timed_runs(f, 1, 2) / 1e3
    out["fused_passes"], out["basic_gates"] = f.plan_stats()
    out["fused_GBps"] = f.last_timings()["bytes"] / out["fused_s"] / 1e9
    if with_plain:
        p = E.Simulation(n, mode="plain", plain_arith="fp64")
        p.extend(circ)
        p.upload()
        p.run()
        out["plain_s"] = p.last_timings()["ms"] / 1e3
        out["plain_GBps"] = p.last_timings()["bytes"] / out["plain_s"] / 1e9
        out["speedup_fused_vs_plain"] = out["plain_s"] / out["fused_s"]
        f.reset_dm()
        f.run()
        out["fused_vs_plain_error"] = f.compare(p)
        p.close()
    if with_oracle:
        out["parity_vs_statevector_oracle"] = oracle_parity(n, circ, f)
    f.close()
    return out


if __name__ == "__main__":
    main()
