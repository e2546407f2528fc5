"""Benchmark: 8-D Gaussian VEGAS events/s, fused fp32 vs plain float64, one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl mine|reference]

Workload (the configuration the metric is quoted on): VegasFlow importance
sampling of prod_d exp(-(x_d-1/2)^2/a^2)/(a sqrt(pi)), a = 0.1, n_dim = 8,
1e8 events per iteration, 50 bins, grid refined every iteration.  One *step* is
one full VEGAS iteration (sample -> map -> evaluate -> reduce -> refine) over
1e8 events.  The headline ``value`` is the fused fp32 form (in-kernel Philox
uniforms, fp32 map/evaluation, compensated sums, float64 across blocks); the
plain float64 path runs the same steps and is reported beside it with both
sigmas (the metric compares them at equal sigma).

Timing: W untimed warm-up iterations, then K timed iterations, each bracketed by
CUDA events on the launching stream; between timed iterations the L2 is flushed
by writing a 512 MB buffer (outside the timed windows).  The iterations draw no
HBM inputs (uniforms come from the in-kernel Philox stream).  Under torchrun
(N > 1) every rank runs an independent replica (different seed), the reported
value is the events of all ranks divided by the slowest rank's time.

``--impl reference`` times the reference algorithm's CPU restatement (the
oracle: TensorFlow is not available on the host) on all host threads: each step
is one whole float64 iteration (refinement included) of one 1e6-event chunk per
thread, a bounded sample of the same workload.  The GPU arm's ``cpu_baseline``
runs the same procedure.
"""

from __future__ import annotations

import argparse
import json
import math
import os
import statistics
import subprocess
import sys
import threading
import time

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, ROOT)

METRIC = "8-D Gaussian events/s, fused FP32 vs plain FP64 at equal σ; served p50/p99"
N_DIM = 8
A_WIDTH = 0.1
EVENTS = 100_000_000
L2_FLUSH_BYTES = 512 << 20
CPU_BASELINE_STEPS = 8  # timed CPU iterations of the GPU arm's cpu_baseline (~10 s on 16 cores)

# Algorithmic instruction budget of one event of the fused fp32 sampler at
# n_dim = 8 (VEGAS map, Gaussian, compensated sums, histogram): counted from the
# algorithm, not from the compiled kernel.
#   Philox4x32-10: 2 blocks x (10 rounds x (2 wide multiplies + 2 three-input xors) + 2)  84
#   map, per dim: not+multiply-add (2), fraction bits (2), fadd, grid load + address (2),
#                 fma (x), fmul (w)                                        9 x 8 =   72
#   Gaussian: 2 fma per dim (16), exp2 (2), prefactor (1)                              19
#   w f, (w f)^2, two TwoSum accumulations (12)                                        14
#   histogram: address + shared atomic per dim                             2 x 8 =   16
#   loop control                                                                        3
INSTR_PER_EVENT_FP32_D8 = 208
# Of those, the 32 x 32 -> 64-bit multiplies (the FMA-heavy pipe, a quarter of
# the FFMA rate on this part): 2 per Philox round x 10 rounds x 2 blocks, and
# one per dimension for the bin map p = 50 w + 25.
WIDE_MUL_PER_EVENT_FP32_D8 = 2 * 10 * 2 + 8

# Injected-uniform mode (uniforms streamed from HBM): algorithmic bytes per event
# = n_dim float64 uniforms.
INJECTED_BYTES_PER_EVENT = 8 * N_DIM

# DRAM traffic of one fp32 sampler launch (grid, parameters; the partial rows stay
# in L2), from one ncu capture of a 1e7-event launch: 40.2 KB read, 0 written.
SAMPLER_DRAM_BYTES = 40192


def _parse():
    ap = argparse.ArgumentParser(description=__doc__, formatter_class=argparse.RawDescriptionHelpFormatter)
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", choices=["mine", "reference"], default="mine")
    ap.add_argument("--events", type=int, default=EVENTS)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--serving-seconds", type=float, default=60.0,
                    help="arrival window of the served Poisson stream (0 = skip)")
    ap.add_argument("--no-precision", action="store_true",
                    help="skip the fp32-versus-float64 comparisons on identical events")
    ap.add_argument("--no-batched", action="store_true", help="skip the 1,024-integral batched run")
    ap.add_argument("--no-injected", action="store_true",
                    help="skip the injected-uniform (HBM-streaming) measurement")
    ap.add_argument("--case", choices=["configs", "c4", "sampler", "injected"],
                    help="run only this workload and print its record (for profiling one kernel family): "
                         "configs = C1 and C3, c4 = the 1,024-integral batch (fp32 only), sampler = "
                         "generate_random_array, injected = streamed float64 uniforms")
    return ap.parse_args()


# ------------------------------------------------------------------ distributed
def dist_setup(n_gpus):
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        backend = "nccl" if torch.cuda.is_available() else "gloo"
        dist.init_process_group(backend=backend)
        if torch.cuda.is_available():
            torch.cuda.set_device(local)
    return rank, world, local


def barrier(world):
    if world > 1:
        import torch.distributed as dist

        dist.barrier()


def max_over_ranks(value, world):
    """The slowest rank's time (replicas: max over ranks)."""
    if world <= 1:
        return value
    import torch
    import torch.distributed as dist

    dev = "cuda" if torch.cuda.is_available() and dist.get_backend() == "nccl" else "cpu"
    t = torch.tensor([float(value)], dtype=torch.float64, device=dev)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


# ------------------------------------------------------------------ clocks
class ClockSampler:
    """nvidia-smi samples (200 ms) during a timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index=0):
        self.gpu = gpu_index
        self.proc = None
        self.lines = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}",
                 "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self._t = threading.Thread(target=self._read, daemon=True)
            self._t.start()
        except (OSError, ValueError):
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc is not None:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        sm, mx, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                mx.append(float(parts[2]))
            except ValueError:
                continue
            for name, val in zip(names, parts[5:9]):
                if val.lower().startswith("active"):
                    reasons.add(name)
        if not sm:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["unavailable"], "samples": 0}
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": max(mx), "reasons": sorted(reasons),
                "samples": len(sm)}


# ------------------------------------------------------------------ reference arm
CPU_CHUNK = 1_000_000  # the reference's default events_limit (configflow.py:22)


class CpuVegas:
    """The float64 VegasFlow iteration of the 8-D Gaussian on the host cores,
    through the oracle (the reference's algorithm restated in NumPy; TensorFlow,
    which the reference runs on, is not installed on the host).  One step is one
    whole iteration of ``threads`` chunks of ``CPU_CHUNK`` events -- one chunk
    per thread, so every thread counted in ``cores`` works -- including the map,
    the integrand, the sums, the histogram and the grid refinement; the grid
    carries over from step to step as in a run of several iterations."""

    def __init__(self, threads):
        import oracle

        self.oracle = oracle
        self.threads = threads
        self.events = threads * CPU_CHUNK
        self.grid = oracle.initial_grid(N_DIM)

    def step(self, seed):
        o = self.oracle
        t0 = time.perf_counter()
        res, sigma, arr = o.threaded_vegas_iteration(
            self.grid, self.events, lambda x: o.integrand_symgauss(x, A_WIDTH), seed, self.threads,
            chunk=CPU_CHUNK)
        self.grid = o.refine_grid(arr, self.grid)
        return time.perf_counter() - t0, res, sigma

    def describe(self, steps):
        return {"kind": "port", "cores": self.threads, "threads_busy": self.threads,
                "sample_events_per_step": self.events,
                "sample": f"{steps} VegasFlow iterations x {self.events:.1e} events of the 8-D Gaussian "
                          f"({self.threads} chunks of {CPU_CHUNK:.0e}, one per host thread), float64 oracle "
                          "(NumPy, PCG64 uniforms through the TECH_CUT affine), grid refined inside the "
                          "timed step"}


def host_threads():
    try:
        return len(os.sched_getaffinity(0))
    except AttributeError:
        return os.cpu_count() or 1


def cpu_baseline_run(steps, warmup, seed0=0):
    """Timed CPU steps: (events/s, seconds per step, CpuVegas)."""
    cpu = CpuVegas(host_threads())
    for w in range(warmup):
        cpu.step(seed0 + 1000 + w)
    times = [cpu.step(seed0 + k)[0] for k in range(steps)]
    return cpu.events * len(times) / sum(times), times, cpu


def run_reference(args, rank, world):
    if rank != 0:
        return
    value, times, cpu = cpu_baseline_run(args.steps, args.warmup)
    line = {
        "impl": "reference", "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": args.gpus,
        "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * sum(times) / len(times),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64",
        "data": "synthetic (NumPy PCG64 uniforms through the TECH_CUT affine)",
        "config": workload_config(args),
        "cpu_baseline": dict(cpu.describe(args.steps), value=value, unit="events/s"),
        "e2e": {"value": value, "unit": "events/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def workload_config(args):
    return {"workload": "8-D Gaussian a=0.1, VegasFlow importance sampling (grid trained every "
                        "iteration), 50 bins, 1e8 events/iteration",
            "n_dim": N_DIM, "events_per_iteration": args.events, "bins": 50,
            "parallelism": f"replicas x{args.gpus}" if args.gpus > 1 else "single GPU",
            "l2": "GPU arm: in-kernel Philox uniforms (no HBM inputs), L2 flushed by a 512 MB write "
                  "between timed iterations; CPU arms: host memory"}


# ------------------------------------------------------------------ GPU arm
def timed_iterations(dev, precision, n_events, K, W, seed, flush, world=1, n_dim=N_DIM):
    """W warm-up + K timed iterations of the n_dim Gaussian (a = 0.1), each
    bracketed by CUDA events on the launching stream with an L2 flush (a write
    of ``flush``) before it; returns the integrator, per-iteration and sampler
    times (s), the history rows and the running average."""
    import numpy as np
    import torch

    from vegasflow_gb300 import VegasFlow, integrands

    stream = torch.cuda.current_stream()
    inst = VegasFlow(n_dim, n_events, verbose=False, precision=precision, seed=seed, device=dev)
    inst.compile(integrands.symgauss(A_WIDTH))
    for _ in range(W):
        inst._run_iteration()
    inst._reset_average()
    torch.cuda.synchronize()
    barrier(world)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True),
           torch.cuda.Event(enable_timing=True)) for _ in range(K)]
    for k in range(K):
        flush.fill_(float(k))
        a, b, c = ev[k]
        a.record(stream)
        inst._fill_partials(train=inst.train)
        b.record(stream)
        inst._end_iteration(train=inst.train)
        c.record(stream)
    torch.cuda.synchronize()
    barrier(world)
    step_ms = [a.elapsed_time(c) for a, b, c in ev]
    samp_ms = [a.elapsed_time(b) for a, b, c in ev]
    hist = inst._workspace()["history"][:K].cpu().numpy()
    avg = inst._workspace()["avg"].cpu().numpy()
    return inst, np.array(step_ms) / 1e3, np.array(samp_ms) / 1e3, hist, avg


def c2_small_run(dev, flush, K=10, W=3, n_events=10_000_000):
    """C2's second size: the 8-D Gaussian at 1e7 events per iteration, fp32
    fused and float64, timed as the headline (10 trained iterations)."""
    exact = math.erf(0.5 / A_WIDTH) ** N_DIM
    out = {"workload": f"8-D Gaussian a=0.1, {n_events:.0e} events/iteration, {K} trained iterations"}
    for prec, seed in (("fp32", 12), ("fp64", 13)):
        _, t, smp, _, avg = timed_iterations(dev, prec, n_events, K, W, seed, flush)
        out[prec] = {"events_per_s": n_events * K / float(t.sum()), "ms_per_iteration": 1e3 * float(t.mean()),
                     "sampler_ms": 1e3 * float(smp.mean()), "mean": float(avg[2]), "sigma": float(avg[3]),
                     "pull_vs_exact": (float(avg[2]) - exact) / float(avg[3])}
    out["fp32_over_fp64"] = out["fp32"]["events_per_s"] / out["fp64"]["events_per_s"]
    return out


def precision_run(dev):
    """fp32 - float64 on identical events, in units of the float64 sigma, per
    configuration.  The float64 side is this project's float64 GPU path (the
    reference's arithmetic, bin for bin; the parity tests pin it to the
    reference's own runs) fed the fp32 form's events: the uniforms its Philox
    words stand for (vf_philox_uniforms), on the fp32 run's grid and event
    layout of that iteration.  C2 compares on the reference's injected uniforms
    instead, beside the reference's own float32 mode (its float64 and float32
    runs recorded under the NumPy stand-in for TensorFlow in
    tests/golden/c2_precision.npz)."""
    import numpy as np
    import torch

    from vegasflow_gb300 import VegasFlow, VegasFlowPlus, integrands
    from vegasflow_gb300 import _native as nat
    from vegasflow_gb300.batch import VegasBatch, c4_specs

    def own_uniforms(seed, call, word3, n, d):
        u = torch.empty((n, d), dtype=torch.float64, device=dev)
        nat.call("vf_philox_uniforms", seed, call, word3, 0, n, d, nat.ptr(u), nat.stream_handle())
        return u

    def summary(pulls):
        p = np.asarray(pulls, dtype=np.float64)
        return {"fp32_minus_fp64_over_sigma": [float(v) for v in p], "max_abs": float(np.max(np.abs(p)))}

    out = {}
    # C1: 4-D Gaussian, 1e6 events, 5 trained iterations
    n, d, seed = 1_000_000, 4, 7
    f32 = VegasFlow(d, n, verbose=False, precision="fp32", seed=seed, device=dev)
    f32.compile(integrands.symgauss(A_WIDTH))
    f64 = VegasFlow(d, n, verbose=False, precision="fp64", seed=seed, device=dev, events_limit=n)
    f64.compile(integrands.symgauss(A_WIDTH))
    pulls = []
    for _ in range(5):
        grid, call = f32.divisions.clone(), f32._call_ctr
        r32, _ = f32._run_iteration()
        f64.divisions.copy_(grid)
        u = own_uniforms(seed, call, call >> 28, n, d)
        f64.set_uniform_source(lambda m, dd, u=u: u)
        r64, s64 = f64._run_iteration()
        pulls.append((float(r32) - float(r64)) / float(s64))
    out["C1"] = summary(pulls)
    # C3: VegasFlowPlus adaptive, 6-D Breit-Wigner x linear, 2e6 events, 3 iterations
    n, d, seed = 2_000_000, 6, 21
    coeffs = np.random.default_rng(3).random(5)
    p32 = VegasFlowPlus(d, n, adaptive=True, verbose=False, precision="fp32", seed=seed, device=dev)
    p32.compile(integrands.breit_wigner(coeffs))
    p64 = VegasFlowPlus(d, n, adaptive=True, verbose=False, precision="fp64", seed=seed, device=dev)
    p64.compile(integrands.breit_wigner(coeffs))
    pulls = []
    for _ in range(3):
        grid, n_ev, start = p32.divisions.clone(), p32.n_ev.clone(), p32._ev_start.clone()
        n_tot, call = int(p32.n_events), p32._call_ctr
        r32, _ = p32._run_iteration()
        p64.divisions.copy_(grid)
        p64.n_ev.copy_(n_ev)
        p64._ev_start.copy_(start)
        p64._n_events, p64._n_ev_stale = n_tot, False
        u = own_uniforms(seed, call, call >> 28, n_tot, d)
        p64.set_uniform_source(lambda m, dd, u=u: u)
        r64, s64 = p64._run_iteration()
        pulls.append((float(r32) - float(r64)) / float(s64))
    out["C3"] = summary(pulls)
    # C4: the first iteration of 16 resolvable batched integrals of at most 2e6 events
    specs = c4_specs()
    picks = [i for i, (dd, nn, f) in enumerate(specs)
             if nn <= 2_000_000 and nn * np.prod(np.asarray(f.params(dd))[dd:] * np.sqrt(np.pi)) >= 100][:16]
    b = VegasBatch([specs[i] for i in picks], seed=11, stream_ids=picks)
    b.run(1)
    first = b.history_host()[:, 0, :]
    pulls = []
    for k, i in enumerate(picks):
        dd, nn, f = specs[i]
        g64 = VegasFlow(dd, nn, verbose=False, precision="fp64", seed=11, device=dev, events_limit=nn)
        g64.compile(f)
        u = own_uniforms(11, 0, i, nn, dd)
        g64.set_uniform_source(lambda m, ddd, u=u: u)
        r64, s64 = g64._run_iteration()
        pulls.append((float(first[k, 0]) - float(r64)) / float(s64))
    out["C4"] = dict(summary(pulls), integrals=len(picks))
    # C2 on the reference's injected uniforms: fused fp32, float64 path, reference float32 mode
    fx = np.load(os.path.join(ROOT, "tests", "golden", "c2_precision.npz"))
    n, iters, floor = int(fx["n_events"]), int(fx["iterations"]), float(fx["raw_floor"])
    h64 = fx["f64/history"]
    got = {}
    for prec in ("fp32", "fp64"):
        rng = np.random.default_rng(int(fx["seed"]))

        def source(m, dd, rng=rng):
            raw = np.maximum(rng.random((m, dd)), floor)
            return torch.as_tensor(raw * ((1.0 - 1e-8) - 1e-8) + 1e-8, device=dev)

        inst = VegasFlow(N_DIM, n, verbose=False, precision=prec, device=dev)
        inst.compile(integrands.symgauss(A_WIDTH))
        inst.set_uniform_source(source)
        got[prec] = np.array([[float(v) for v in inst._run_iteration()] for _ in range(iters)])
    out["C2"] = {"events": n, "iterations": iters,
                 "fused_fp32_minus_reference_fp64_over_sigma": [float(v) for v in (got["fp32"][:, 0] - h64[:, 0])
                                                                 / h64[:, 1]],
                 "reference_fp32_mode_minus_fp64_over_sigma": [float(v) for v in (fx["f32/history"][:, 0]
                                                                                   - h64[:, 0]) / h64[:, 1]],
                 "gpu_fp64_minus_reference_fp64_relative": float(np.max(np.abs(got["fp64"][:, 0] - h64[:, 0])
                                                                        / np.abs(h64[:, 0])))}
    return out


def main():
    args = _parse()
    rank, world, local = dist_setup(args.gpus)
    if args.impl == "reference":
        run_reference(args, rank, world)
        return

    import numpy as np
    import torch

    from vegasflow_gb300 import VegasFlow, integrands
    from vegasflow_gb300 import _native as nat
    from vegasflow_gb300.build import build

    build()
    assert torch.cuda.is_available(), "bench.py needs a CUDA GPU"
    dev = torch.device("cuda", local)
    torch.cuda.set_device(dev)
    stream = torch.cuda.current_stream()
    flush = torch.empty(L2_FLUSH_BYTES // 4, dtype=torch.float32, device=dev)
    exact = math.erf(0.5 / A_WIDTH) ** N_DIM
    K, W = args.steps, max(3, args.warmup)
    if args.case:
        run_case = {"configs": lambda: configs_run(dev), "c4": lambda: batched_run(dev, fp64_sample=False),
                    "sampler": lambda: sampler_run(dev, args.events, K, W),
                    "injected": lambda: injected_run(dev, args.events, K, W)}[args.case]
        if rank == 0:
            print(json.dumps({"case": args.case, "result": run_case()}), flush=True)
        return

    def timed_run(precision, seed):
        return timed_iterations(dev, precision, args.events, K, W, seed, flush, world)

    with ClockSampler(local) as clocks:
        inst32, t32, s32, h32, a32 = timed_run("fp32", seed=2 + 1000 * rank)
        inst64, t64, s64, h64, a64 = timed_run("fp64", seed=3 + 1000 * rank)

        # issue-rate calibration at the same clocks
        probe_blocks = 152 * 8
        probe_buf = torch.empty(probe_blocks * 256, dtype=torch.float32, device=dev)
        import ctypes
        fpt = ctypes.c_longlong(0)
        lib = nat.load()
        for _ in range(2):
            nat.check(lib.vf_issue_probe(nat.ptr(probe_buf), probe_blocks, 4000, ctypes.byref(fpt),
                                         nat.stream_handle()))
        pa, pb = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pa.record(stream)
        nat.check(lib.vf_issue_probe(nat.ptr(probe_buf), probe_blocks, 4000, ctypes.byref(fpt),
                                     nat.stream_handle()))
        pb.record(stream)
        torch.cuda.synchronize()
        probe_s = pa.elapsed_time(pb) / 1e3
        issue_peak = probe_blocks * 256 * fpt.value / 32 / probe_s  # warp instructions / s
        # the FMA-heavy pipe's rate for the 64-bit multiplies of Philox and the bin map
        mul_buf = probe_buf.view(torch.int32)
        mpt = ctypes.c_longlong(0)
        for _ in range(2):
            nat.check(lib.vf_widemul_probe(nat.ptr(mul_buf), probe_blocks, 4000, ctypes.byref(mpt),
                                           nat.stream_handle()))
        pa.record(stream)
        nat.check(lib.vf_widemul_probe(nat.ptr(mul_buf), probe_blocks, 4000, ctypes.byref(mpt),
                                       nat.stream_handle()))
        pb.record(stream)
        torch.cuda.synchronize()
        widemul_peak = probe_blocks * 256 * mpt.value / 32 / (pa.elapsed_time(pb) / 1e3)  # warp instr / s

        # end to end with host buffers: through the C-ABI as a plugin drives it
        # (the headline), and through the Python API
        e2e = e2e_abi_run(dev, args.events, K, W, seed=21 + 1000 * rank)
        e2e_api = e2e_run(inst32, K, dev)
        injected = None if args.no_injected else injected_run(dev, args.events, K, W)
        sampler = None if args.no_injected else sampler_run(dev, args.events, K, W)
        configs = None if args.no_batched else configs_run(dev)
        c2_small = c2_small_run(dev, flush) if args.events == EVENTS and not args.no_batched else None
    clk = clocks.summary()

    total32 = float(t32.sum())
    total32 = max_over_ranks(total32, world)
    total64 = max_over_ranks(float(t64.sum()), world)
    events_all = args.events * K * world
    value = events_all / total32
    value64 = events_all / total64

    samp_mean = float(s32.mean())
    line = {
        "metric": METRIC, "value": value, "unit": "events/s", "n_gpus": world, "steps": K, "warmup": W,
        "ms_per_step": 1e3 * total32 / K, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32",
        "data": "synthetic (in-kernel Philox4x32-10 uniforms)",
        "config": workload_config(args),
        "result": {"fp32": {"mean": float(a32[2]), "sigma": float(a32[3]), "chi2_dof": float(a32[4]),
                            "pull_vs_exact": (float(a32[2]) - exact) / float(a32[3])},
                   "fp64": {"mean": float(a64[2]), "sigma": float(a64[3]), "chi2_dof": float(a64[4]),
                            "pull_vs_exact": (float(a64[2]) - exact) / float(a64[3])},
                   "exact": exact},
        "fp64_plain": {"value": value64, "unit": "events/s", "ms_per_step": 1e3 * total64 / K,
                       "sampler_ms": 1e3 * float(s64.mean())},
        "fp32_over_fp64": value / value64,
        "roofline": sampler_roofline(args.events / samp_mean, samp_mean, issue_peak, widemul_peak),
        "e2e": e2e,
        "e2e_python_api": e2e_api,
        "injected": injected,
        "sampler": sampler,
        "configs": configs,
        "c2_1e7": c2_small,
        "gpu_launches": 2 * K,
        "clocks": clk,
    }
    if not args.no_batched:
        line["batched"] = batched_run(dev)
    if not args.no_precision:
        line["precision"] = precision_run(dev)
    if args.serving_seconds > 0:
        line["serving"] = serving_run(args.serving_seconds)
    if rank == 0 and world == 1 and not args.no_cpu_baseline:
        rate, times, cpu = cpu_baseline_run(CPU_BASELINE_STEPS, 1)
        line["cpu_baseline"] = dict(cpu.describe(len(times)), value=rate, unit="events/s",
                                    seconds=float(sum(times)))
    if rank == 0:
        print(json.dumps(line), flush=True)
    if world > 1:
        import torch.distributed as dist

        dist.destroy_process_group()


def sampler_roofline(events_per_s, sampler_s, issue_peak, widemul_peak):
    """The headline kernel's roofline: the binding pipe of its per-event
    instruction budget (the lower of the pipe bounds), both pipes measured in
    this run.  `achieved` = the event's instructions on that pipe x events / 32
    / sampler time, against the pipe's probe rate."""
    bounds = pipe_bounds(events_per_s, issue_peak, widemul_peak)
    b = bounds["binding"]
    ops = bounds[b]["ops_per_event"]
    peak = bounds[b]["peak_gwarp_instr_per_s"] * 1e9
    achieved = ops * events_per_s / 32
    names = {"issue": ("issue (warp-instruction issue rate)", "vf_issue_probe: independent FFMA chains"),
             "fma_heavy_wide_multiplies": ("FMA-heavy pipe (64-bit integer multiplies of Philox and the bin map)",
                                           "vf_widemul_probe: Philox-shaped multiply/XOR chains")}
    return {"bound": names[b][0], "kernel": "vf_vegas_f32_kernel<8,SYMGAUSS,1024>",
            "achieved": achieved / 1e9, "peak": peak / 1e9, "unit": "Gwarp-instr/s", "frac": achieved / peak,
            "traffic": SAMPLER_DRAM_BYTES,
            "traffic_note": "DRAM bytes per launch (ncu dram__bytes_read.sum + dram__bytes_write.sum on a "
                            "1e7-event launch); the kernel streams no per-event data, so this does not grow "
                            "with events",
            "per_event_instr": ops,
            "peak_source": "measured in this run: " + names[b][1],
            "pipe_bounds": bounds,
            "sampler_ms": 1e3 * sampler_s}


def pipe_bounds(events_per_s, issue_peak, widemul_peak):
    """The fused sampler's per-pipe bounds at D = 8, each from a rate measured
    in this run: events/s if only that pipe limited it (its peak warp
    instructions/s x 32 / the event's instructions on it), and the sampler's
    fraction of each.  Issue: all 208 algorithmic instructions; the FMA-heavy
    pipe: the 48 64-bit multiplies (40 in the two Philox blocks, 8 in the bin
    map), at the rate of vf_widemul_probe."""
    ev_s = events_per_s
    out = {}
    for name, peak, ops in (("issue", issue_peak, INSTR_PER_EVENT_FP32_D8),
                            ("fma_heavy_wide_multiplies", widemul_peak, WIDE_MUL_PER_EVENT_FP32_D8)):
        bound = peak * 32 / ops
        out[name] = {"ops_per_event": ops, "peak_gwarp_instr_per_s": peak / 1e9,
                     "bound_events_per_s": bound, "frac": ev_s / bound}
    out["binding"] = min(("issue", "fma_heavy_wide_multiplies"), key=lambda k: out[k]["bound_events_per_s"])
    return out


def measured_hbm_peak():
    """(GB/s, source) from MEASURED_PEAKS.json, else the fallback figure."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["hbm_gbs"]), "measured (MEASURED_PEAKS.json hbm_gbs)"
    except (OSError, ValueError, KeyError):
        return 6800.0, "fallback 6.8 TB/s"


def injected_run(dev, n_events, K, W, seed=11):
    """C2 injected mode: the float64 uniforms of every event (n x 8 x 8 bytes,
    6.4 GB at 1e8) resident in HBM and streamed once per iteration by the fused
    fp32 sampler (TMA tiles), the grid trained every iteration.  The array is far
    larger than L2, so every iteration reads it from HBM."""
    import torch

    from vegasflow_gb300 import VegasFlow, integrands

    inst = VegasFlow(N_DIM, n_events, verbose=False, precision="fp32", seed=seed, device=dev)
    inst.compile(integrands.symgauss(A_WIDTH))
    for _ in range(2):  # a trained grid
        inst._run_iteration()
    gen = torch.Generator(device=dev)
    gen.manual_seed(seed)
    tc = 1e-8  # the reference's TECH_CUT affine: U[tc, 1 - tc)
    u = torch.rand((n_events, N_DIM), dtype=torch.float64, device=dev, generator=gen)
    u.mul_(1.0 - 2.0 * tc).add_(tc)
    stream = torch.cuda.current_stream()

    def step(call, marks=None):
        if marks:
            marks[0].record(stream)
        inst._sample(n_events, 0, call, inst._int_id, inst._params_dev, True, False, u_inj=u)
        if marks:
            marks[1].record(stream)
        inst._end_iteration(train=True)
        if marks:
            marks[2].record(stream)

    for w in range(W):
        step(w)
    inst._reset_average()
    marks = [[torch.cuda.Event(enable_timing=True) for _ in range(3)] for _ in range(K)]
    torch.cuda.synchronize()
    for k in range(K):
        step(100 + k, marks[k])
    torch.cuda.synchronize()
    step_ms = [a.elapsed_time(c) for a, b, c in marks]
    samp_ms = [a.elapsed_time(b) for a, b, c in marks]
    first = inst._workspace()["history"][0].cpu().numpy()
    flags = int(inst._workspace()["flags"][0].item())
    del u
    torch.cuda.empty_cache()
    samp = statistics.mean(samp_ms) / 1e3
    achieved = INJECTED_BYTES_PER_EVENT * n_events / samp / 1e9
    peak, source = measured_hbm_peak()
    exact = math.erf(0.5 / A_WIDTH) ** N_DIM
    return {
        "workload": f"C2 injected mode: {n_events:.0e} float64 uniforms x {N_DIM} resident in HBM "
                    f"({INJECTED_BYTES_PER_EVENT * n_events / 1e9:.1f} GB, larger than L2), fused fp32 "
                    "sampler + iteration end, grid trained",
        "value": K * n_events / (sum(step_ms) / 1e3), "unit": "events/s",
        "ms_per_step": statistics.mean(step_ms), "sampler_ms": 1e3 * samp,
        # every iteration replays the same uniforms, so only one iteration is an
        # independent estimate
        "first_timed_iteration": {"mean": float(first[0]), "sigma": float(first[1]),
                                  "pull_vs_exact": (float(first[0]) - exact) / float(first[1])},
        "flags": flags,
        "roofline": {"bound": "hbm", "kernel": "vf_vegas_f32_inj_kernel<8,SYMGAUSS> (TMA stage rings)",
                     "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "traffic": INJECTED_BYTES_PER_EVENT * n_events,
                     "traffic_note": "algorithmic bytes; ncu dram__bytes (read + write) on a 1e7-event "
                                     "launch equals them to within 1%",
                     "peak_source": source},
    }


def sampler_run(dev, n_events, K, W, seed=3):
    """The sampler API (VEGAS as a random-number generator): on a trained
    8-D grid, ``generate_random_array(n)`` writes x (8 floats) and the
    normalised weight (1 float) of every event to HBM -- one map kernel launch.
    ``value`` is through the public call; the roofline is the map kernel alone
    (36 bytes written per event)."""
    import torch

    from vegasflow_gb300 import VegasFlow, integrands
    from vegasflow_gb300 import _native as nat

    inst = VegasFlow(N_DIM, n_events, verbose=False, precision="fp32", seed=seed, device=dev)
    inst.compile(integrands.symgauss(A_WIDTH))
    for _ in range(2):
        inst._run_iteration()
    stream = torch.cuda.current_stream()
    x = torch.empty((n_events, N_DIM), dtype=torch.float32, device=dev)
    w = torch.empty(n_events, dtype=torch.float32, device=dev)
    for k in range(W):
        inst.generate_random_array(n_events)
        inst._sample(n_events, 0, 900 + k, nat.VF_INT_NONE, None, False, False, x=x, w=w)
    torch.cuda.synchronize()
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record(stream)
    for k in range(K):
        xr, pr = inst.generate_random_array(n_events)
    b.record(stream)
    b.synchronize()
    api_ms = a.elapsed_time(b) / K
    del xr, pr
    a.record(stream)
    for k in range(K):
        inst._sample(n_events, 0, 950 + k, nat.VF_INT_NONE, None, False, False, x=x, w=w)
    b.record(stream)
    b.synchronize()
    kern_ms = a.elapsed_time(b) / K
    del x, w
    torch.cuda.empty_cache()
    bytes_per_event = 4 * N_DIM + 4
    achieved = bytes_per_event * n_events / (kern_ms / 1e3) / 1e9
    peak, source = measured_hbm_peak()
    return {
        "workload": f"generate_random_array({n_events:.0e}) on a trained {N_DIM}-D grid, fp32 x and weight",
        "value": n_events / (api_ms / 1e3), "unit": "events/s", "ms_per_call": api_ms, "kernel_ms": kern_ms,
        "roofline": {"bound": "hbm", "kernel": "vf_vegas_f32_map_kernel<8,false>", "achieved": achieved, "peak": peak,
                     "unit": "GB/s", "frac": achieved / peak, "traffic": bytes_per_event * n_events,
                     "traffic_note": "algorithmic bytes written (x 32 B + w 4 B per event)",
                     "peak_source": source},
    }


def configs_run(dev):
    """The other configurations of the metric, briefly: C1 (4-D Gaussian,
    float64, 1e6 events x 5 iterations, seed 7) and C3 (VegasFlowPlus adaptive,
    6-D Breit-Wigner x linear, 2e6 events x 10 iterations) in both precisions,
    each against its exact value, with eager iterations and with CUDA-graph
    replays (``cuda_graph=True``); ``events_per_s`` is the faster of the two."""
    import numpy as np
    import torch

    from vegasflow_gb300 import VegasFlow, VegasFlowPlus, integrands

    out = {}
    exact1 = math.erf(0.5 / A_WIDTH) ** 4
    coeffs = np.random.default_rng(3).random(5)
    exact3 = integrands.breit_wigner_exact(6, coeffs)
    for name, make, it, exact in (
            ("C1", lambda p, g: (VegasFlow(4, 1_000_000, verbose=False, precision=p, seed=7, device=dev,
                                           cuda_graph=g), integrands.symgauss(A_WIDTH)), 5, exact1),
            ("C3", lambda p, g: (VegasFlowPlus(6, 2_000_000, adaptive=True, verbose=False, precision=p, seed=7,
                                               device=dev, cuda_graph=g), integrands.breit_wigner(coeffs)),
             10, exact3)):
        for prec in ("fp64", "fp32"):
            row = {}
            for graph in (False, True):
                inst, f = make(prec, graph)
                inst.compile(f)
                inst.run_integration(it)  # warm-up: compile-time work, first launches, the graph capture
                n0 = inst.n_events
                torch.cuda.synchronize()
                t0 = time.perf_counter()
                res, sig = inst.run_integration(it)
                dt = time.perf_counter() - t0
                # VegasFlowPlus reallocates every iteration: the mean of the counts before and after
                events = it * (n0 + inst.n_events) / 2
                key = "graph" if graph else "eager"
                row[key] = {"events_per_s": events / dt, "seconds": dt, "mean": float(res), "sigma": float(sig),
                            "pull_vs_exact": (float(res) - exact) / float(sig)}
            best = max(row, key=lambda k: row[k]["events_per_s"])
            out[f"{name}_{prec}"] = dict(row[best], iterations=best, eager_events_per_s=row["eager"]["events_per_s"],
                                         graph_events_per_s=row["graph"]["events_per_s"])
    return out


def batched_run(dev, n_iter=5, fp64_sample=True):
    """C4: 1,024 Gaussians (dims 2-16, 1e4-1e7 events) with their own grids, 5
    iterations as CUDA-graph replays of the batched fp32 engine, against the
    float64 single-integral path run one integral after another on a sample."""
    import numpy as np
    import torch

    from vegasflow_gb300 import VegasFlow
    from vegasflow_gb300.batch import VegasBatch, c4_specs

    specs = c4_specs()
    b = VegasBatch(specs, seed=11)
    b.run(1, graph=True)
    b.reset_average()
    torch.cuda.synchronize()
    a, c = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    a.record()
    b.run(n_iter, graph=True)
    c.record()
    torch.cuda.synchronize()
    t = a.elapsed_time(c) / 1e3
    ev = b.total_events() * n_iter
    # pulls against the exact integrals, over the integrals VEGAS can resolve at
    # these sizes (>= 100 expected events in the peak on the initial grid)
    from vegasflow_gb300.integrands import gauss_exact

    mean, sigma, _, flags = b.results()
    pulls = []
    for i, (d, n, f) in enumerate(specs):
        p = np.asarray(f.params(d))
        if n * np.prod(p[d:] * np.sqrt(np.pi)) >= 100 and np.isfinite(mean[i]) and sigma[i] > 0:
            pulls.append((mean[i] - gauss_exact(p[:d], p[d:])) / sigma[i])
    pulls = np.asarray(pulls)
    out = {"workload": "1,024 Gaussians, dims 2-16, 1e4-1e7 events/iteration, own grids, 5 iterations",
           "integrals": len(specs), "events_per_iteration": b.total_events(),
           "fp32_batched_events_per_s": ev / t, "ms_per_iteration": 1e3 * t / n_iter,
           "graph": True, "launches_per_iteration": 2,
           "pulls_vs_exact": {"resolvable": int(pulls.size), "mean": float(pulls.mean()),
                              "rms": float(np.sqrt(np.mean(pulls ** 2))),
                              "within_3_sigma": float(np.mean(np.abs(pulls) < 3.0))},
           "flags": int(flags)}
    if not fp64_sample:
        return out
    # float64 one by one, on every 16th integral (64 of them)
    sample = specs[::16]
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for d, n, f in sample:
        inst = VegasFlow(d, n, verbose=False, precision="fp64", seed=11, device=dev)
        inst.compile(f)
        inst.run_integration(n_iter)
    torch.cuda.synchronize()
    t64 = time.perf_counter() - t0
    ev64 = sum(n for _, n, _ in sample) * n_iter
    out.update({"fp64_one_by_one_events_per_s": ev64 / t64,
                "fp64_sample": f"{len(sample)} of the 1,024 integrals, run_integration({n_iter}) each"})
    return out


def serving_run(seconds):
    """C5: Poisson arrivals at 200/s (seed 9), 20% Breit-Wigner, target relative
    sigma 1e-3, at most 20 iterations, 150 GB admission budget, real time."""
    from vegasflow_gb300.serving import VegasServer, poisson_workload

    reqs = poisson_workload(rate=200.0, duration=seconds, seed=9)
    server = VegasServer(max_slots=4096, hbm_budget=150e9, seed=9)
    m = server.run(reqs, realtime=True)
    m["arrival_window_s"] = seconds
    m["rate_per_s"] = 200.0
    return m


def e2e_abi_run(dev, n_events, K, W, seed):
    """The headline workload end to end through the C-ABI with host buffers, as a
    plugin binding ``libvegasgb.so`` drives it: the plugin allocates its device
    buffers once; per step one cudaMemcpyAsync of the grid from pinned host
    memory, one ``vf_iteration_dev`` call (the fused fp32 sampler and the
    iteration end: one VegasFlow iteration with float32 refinement), one
    cudaMemcpyAsync of the refined grid, the (result, sigma) rows and the flags
    word back into pinned host memory, and one stream synchronize.  Host clock
    around the K steps (after W untimed ones)."""
    import ctypes

    import numpy as np
    import torch

    from vegasflow_gb300 import _native as nat

    lib = nat.load()
    d, cap = N_DIM, K + W
    rows = ctypes.c_int(0)
    nat.check(lib.vf_sample_rows(nat.VF_ALG_VEGAS, nat.VF_PREC_F32, d, nat.VF_INT_SYMGAUSS, 1,
                                 ctypes.byref(rows)))
    ng = d * 51
    nd = ng + 2 * cap + 1  # the grid, the history rows, the flags word (in a float64 slot)
    dev_buf = torch.zeros(nd, dtype=torch.float64, device=dev)
    host = torch.zeros(nd, dtype=torch.float64).pin_memory()
    host[:ng] = torch.linspace(0.0, 1.0, 51, dtype=torch.float64).repeat(d)
    grid, hist = dev_buf[:ng], dev_buf[ng:ng + 2 * cap]
    flags = dev_buf[ng + 2 * cap:].view(torch.int32)[:1]
    partials = torch.empty(rows.value * (2 + 50 * d), dtype=torch.float64, device=dev)
    avg = torch.zeros(5, dtype=torch.float64, device=dev)
    counters = torch.zeros(2, dtype=torch.int32, device=dev)
    params = torch.tensor([A_WIDTH, (1.0 / A_WIDTH / math.sqrt(math.pi)) ** d], dtype=torch.float64, device=dev)
    stream = torch.cuda.current_stream()
    sh = nat.stream_handle()
    torch.cuda.synchronize()

    def step():
        grid.copy_(host[:ng], non_blocking=True)
        nat.call("vf_iteration_dev", nat.VF_ALG_VEGAS, nat.VF_PREC_F32, nat.ptr(grid), d, n_events,
                 1.0 / n_events, None, None, 1.0, seed, nat.ptr(counters[0:1]), nat.ptr(counters[1:2]),
                 nat.VF_INT_SYMGAUSS, nat.ptr(params), 1, 1.5, nat.ptr(partials), rows.value, nat.ptr(hist),
                 cap, nat.ptr(avg), nat.ptr(flags), sh)
        host.copy_(dev_buf, non_blocking=True)
        stream.synchronize()

    for _ in range(W):
        step()
    t0 = time.perf_counter()
    for _ in range(K):
        step()
    dt = time.perf_counter() - t0
    res = host[ng:ng + 2 * cap].view(cap, 2).numpy()
    flag_word = int(host[ng + 2 * cap:].numpy().view(np.int32)[0])
    exact = math.erf(0.5 / A_WIDTH) ** d
    last = res[cap - 1]
    del dev_buf, partials
    return {"value": n_events * K / dt, "unit": "events/s", "h2d_bytes_per_step": ng * 8,
            "d2h_bytes_per_step": nd * 8, "ms_per_step": 1e3 * dt / K,
            "api": "C-ABI: per step cudaMemcpyAsync H2D of the grid (pinned host), vf_iteration_dev, "
                   "cudaMemcpyAsync D2H of grid + result rows + flags, stream synchronize",
            "last_iteration": {"result": float(last[0]), "sigma": float(last[1]),
                               "pull_vs_exact": (float(last[0]) - exact) / float(last[1])},
            "flags": flag_word}


def e2e_run(inst, K, dev):
    """K steps through the public API (``run_integration(1)`` per step) with the
    grid kept in pinned host memory: per step H2D of the grid, the iteration and
    the D2H read of its (result, sigma), then D2H of the refined grid."""
    import torch

    host_grid = inst.divisions.cpu().pin_memory()
    for _ in range(2):
        inst.divisions.copy_(host_grid, non_blocking=True)
        inst.run_integration(1)
        host_grid.copy_(inst.divisions, non_blocking=True)
        torch.cuda.current_stream().synchronize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for _ in range(K):
        inst.divisions.copy_(host_grid, non_blocking=True)
        inst.run_integration(1)
        host_grid.copy_(inst.divisions, non_blocking=True)
        torch.cuda.current_stream().synchronize()
    dt = time.perf_counter() - t0
    nbytes = host_grid.numel() * 8
    return {"value": inst.n_events * K / dt, "unit": "events/s", "h2d_bytes_per_step": nbytes,
            "d2h_bytes_per_step": nbytes + 16 + 5 * 8 + 8,
            "api": "VegasFlow.run_integration(1) per step, grid resident in pinned host memory"}


if __name__ == "__main__":
    main()
