"""Benchmark of the FDTD hot path on GB300.

Default workload (the headline): the 2D TM PML benchmark program -- 8192x8192
grid, 32-cell PML with cubic grading 0.333, lossy dielectric cylinder of radius
1000 cells (eps_r=30, sigma=0.3 S/m), hard Gaussian Dz source at the centre
(t0=20, spread=6), 2000 time steps, FP32.  One bench "step" = one complete
2000-step simulation from zero fields (1.342e11 cell-updates).

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]

Prints ONE JSON line (rank 0).  ``value`` is Gcell-updates/s over all ranks
with inputs resident in HBM; ``e2e`` is the same metric through the public API
with host buffers (pinned host -> device copies of the initial fields and
material map, and device -> host copies of all seven result fields, inside the
timed region).  Under torchrun each rank runs an independent replica (the 2D
update does not shard on one node here: replicas only), value = total.

``--impl reference`` times the reference's CPU path (the C restatement of
fd2d/clang/test_3_4.c's loops, float32, OpenMP on all host cores; the
reference's own C cannot be built on the GPU host) on a bounded sample of the
same workload.
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
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

NX = NY = 8192
NPML = 32
GRADE = 0.333
RGRID = 1000
EPSR, SIGMA = 30.0, 0.3
NS = 2000
E2E_MIN_STEPS = 6  # requests in the end-to-end run (amortises the pipeline fill and drain)
BYTES_PER_CELL_UPDATE = 60  # lossy PML update: 8 float reads + 7 float writes per cell
METRIC = "Gcell-updates/s & %HBM peak; surrogate vs FDTD spectra/s at ≤1% L2 error"
UNIT = "Gcell-updates/s"
WORKLOAD = ("2D TM PML lossy-cylinder benchmark program: 8192x8192, npml=32 grade 0.333, "
            "cylinder r=1000 eps_r=30 sigma=0.3, hard Gaussian Dz source t0=20 spread=6, 2000 steps, FP32")
# DRAM bytes per cell per fused K=4 pass, from one ncu capture of the fused kernel
# on the 4096^2 case ((dram__bytes_read.sum + dram__bytes_write.sum) / cells =
# 1009.4 MB / 16.78 M cells, profiles/k_march_K4_CPL4_full_4096.md); traffic
# grows in proportion to the cells, so it is scaled to the launch size
NCU_TRAFFIC_BYTES_PER_CELL_PASS = {4: 60.2}


def _peaks():
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    try:
        with open(p) as fh:
            d = json.load(fh)
        return float(d["hbm_gbs"]), "measured"
    except Exception:
        return 6800.0, "fallback"


def _peaks_bf16():
    """Dense BF16 TFLOP/s measured as a burst (the surrogate pass is timed alone)."""
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as fh:
            return float(json.load(fh)["bf16_tflops"])
    except Exception:
        return 1900.0


class Clocks:
    """nvidia-smi sampling during the timed region."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int):
        self.index = index
        self.proc = None
        self.path = None

    def start(self):
        try:
            fd, self.path = tempfile.mkstemp(suffix=".csv")
            os.close(fd)
            self.fh = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=self.fh, stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self) -> dict:
        if self.proc is None:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.fh.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        with open(self.path) as fh:
            for line in fh:
                f = [x.strip() for x in line.split(",")]
                if len(f) < 9:
                    continue
                try:
                    sm.append(float(f[1]))
                    smax.append(float(f[2]))
                except ValueError:
                    continue
                for n, v in zip(names, f[5:9]):
                    if v.lower().startswith("active"):
                        reasons.add(n)
        os.unlink(self.path)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm)}


_CPU_SETUP = {}


def _cpu_setup(nx: int, ny: int):
    """Material map and PML of the benchmark program for the C port (cached)."""
    import numpy as np

    from oracle import fd2d as O
    key = (nx, ny)
    if key not in _CPU_SETUP:
        dt = 0.01 / 6e8
        pml = O.pmlparam(nx, ny, NPML, GRADE)
        naz = np.ones((nx, ny), dtype=np.float32)
        nbz = np.zeros((nx, ny), dtype=np.float32)
        for r0 in range(0, nx, 512):  # material map in row bands (float64 formula)
            a, b = O.dielectric(nx, ny, NPML, RGRID, dt, EPSR, SIGMA, rows=slice(r0, min(nx, r0 + 512)))
            naz[r0:r0 + a.shape[0]] = a
            nbz[r0:r0 + b.shape[0]] = b
        pd = {k: getattr(pml, k) for k in ("fx1", "fx2", "fx3", "fy1", "fy2", "fy3", "gx2", "gx3", "gy2", "gy3")}
        _CPU_SETUP[key] = (pd, naz, nbz)
    return _CPU_SETUP[key]


def host_cpu() -> str:
    """The host CPU's model as lscpu reports it (with its core count)."""
    try:
        out = subprocess.run(["lscpu"], capture_output=True, text=True, timeout=10).stdout
        d = dict(line.split(":", 1) for line in out.splitlines() if ":" in line)
        name = (d.get("Model name") or d.get("Vendor ID") or "unknown").strip()
        return f"{name}, {os.cpu_count()} logical CPUs, {(d.get('Architecture') or '').strip()}"
    except Exception:
        return f"unknown, {os.cpu_count()} logical CPUs"


def cpu_port_rate(nx: int, ny: int, steps: int, threads: int | None = None, native: bool = False) -> dict:
    """Time the float32 OpenMP C port of the reference loops on this host:
    the portable -O3 build, or (native) the build tuned for this host's CPU."""
    import numpy as np

    from oracle import ccore
    lib = ccore.lib32_native() if native else ccore.lib32()
    if lib is None:
        return {"value": 0.0, "seconds": 0.0, "cores": 0, "sample": "native build unavailable"}
    if threads:
        lib.oracle_set_threads(threads)
    else:
        lib.oracle_set_threads(os.cpu_count() or 1)
    nth = lib.oracle_threads()
    pd, naz, nbz = _cpu_setup(nx, ny)
    f = {k: np.zeros((nx, ny), dtype=np.float32) for k in ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy")}
    table = np.exp(-0.5 * ((np.arange(1, steps + 2) - 20) / 6.0) ** 2)
    ccore.fd2d_steps(lib, np.float32, nx, ny, 0, 1, pd, naz, nbz, (1, nx // 2, ny // 2), table, f)  # warm-up
    t0 = time.perf_counter()
    ccore.fd2d_steps(lib, np.float32, nx, ny, 1, steps, pd, naz, nbz, (1, nx // 2, ny // 2), table, f)
    el = time.perf_counter() - t0
    flags = "-O3 -march/-mcpu=native" if native else "-O3"
    return {"value": nx * ny * steps / el / 1e9, "seconds": el, "cores": nth, "build": f"gcc {flags} -fopenmp",
            "sample": f"{nx}x{ny} grid, {steps} steps of the same lossy PML update (float32 C port, OpenMP)"}


def cpu_best_rate(nx: int, ny: int, steps: int, threads: int | None = None) -> dict:
    """The faster of the portable and the host-tuned builds of the float32
    port (the other one's rate is kept beside it), with the host CPU named."""
    a = cpu_port_rate(nx, ny, steps, threads)
    b = cpu_port_rate(nx, ny, steps, threads, native=True)
    best, other = (b, a) if b["value"] > a["value"] else (a, b)
    best = dict(best)
    best["other_build"] = {"build": other.get("build"), "value": other["value"]}
    best["cpu"] = host_cpu()
    return best


def max_over_ranks(ms: float, world: int, device) -> float:
    """The slowest rank's time: replicas finish when the last one does."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(cell_updates_per_rank: int, world: int, ms: float) -> float:
    """Gcell-updates/s of the whole job: every rank's work over the slowest time."""
    return cell_updates_per_rank * world / (ms / 1e3) / 1e9


def numpy_reference_rate(n: int = 2048, steps: int = 10) -> dict:
    """Time the reference's own NumPy form of the step (the oracle's float64
    restatement of fd2d/program/fd2d_3_2.py:61-93 with the lossy efield of
    fd2d/python/fd2d_3_4.py:131-136) on a bounded sample, one host thread."""
    from oracle import fd2d as O
    dt = 0.01 / 6e8
    pml = O.pmlparam(n, n, NPML, GRADE)
    naz, nbz = O.dielectric(n, n, NPML, n // 8, dt, EPSR, SIGMA)
    src = ("hard", n // 2, n // 2, ("gauss", 20, 6.0))
    st = O.run(n, n, 1, pml=pml, naz=naz, nbz=nbz, src=src)  # warm-up step
    t0 = time.perf_counter()
    O.run(n, n, steps, pml=pml, naz=naz, nbz=nbz, src=src, state=st, t_start=2)
    el = time.perf_counter() - t0
    return {"value": n * n * steps / el / 1e9, "seconds": el, "cores": 1,
            "sample": f"{n}x{n} grid, {steps} steps of the float64 NumPy form of the reference step"}


def run_reference(args) -> None:
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    import numpy as np  # noqa: F401
    steps_per_sample = int(os.environ.get("FDTD_REF_SAMPLE_STEPS", "20"))
    for _ in range(args.warmup):
        cpu_port_rate(NX, NY, 1)
    # the faster of the two builds on this host, then the timed samples with it
    native = cpu_port_rate(NX, NY, 2, native=True)["value"] > cpu_port_rate(NX, NY, 2)["value"]
    vals = []
    for _ in range(args.steps):
        r = cpu_port_rate(NX, NY, steps_per_sample, native=native)
        vals.append(r)
    tot_cells = sum(NX * NY * steps_per_sample for _ in vals)
    tot_s = sum(v["seconds"] for v in vals)
    value = tot_cells / tot_s / 1e9
    line = {"impl": "reference", "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1e3 * tot_s / len(vals),
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32",
            "data": "synthetic (deterministic benchmark program, no RNG)",
            "config": {"workload": WORKLOAD, "sample_steps_per_step": steps_per_sample, "grid": [NX, NY]},
            "cpu_baseline": {"value": value, "unit": UNIT, "cores": vals[0]["cores"], "kind": "port",
                             "sample": vals[0]["sample"], "build": vals[0]["build"], "cpu": host_cpu()},
            "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def run_ours(args) -> None:
    import torch
    import torch.distributed as dist

    from simulation_gb300 import fd2d as G

    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        dist.init_process_group("nccl")
    torch.cuda.set_device(local)
    dev = torch.device("cuda", local)

    def barrier():
        if world > 1:
            dist.barrier()
        torch.cuda.synchronize()

    sim = G.benchmark_sim(NX, NY, NPML, GRADE, RGRID, EPSR, SIGMA, ns=NS, device=dev,
                          steps_per_pass=args.spp)
    spp = args.spp
    cells = NX * NY
    passes_per_run = -(-NS // spp)
    passes_per_run += passes_per_run % 2

    def one_run():
        sim.reset()
        sim.step(NS)

    for _ in range(max(args.warmup, 3)):
        one_run()
    barrier()
    clk = Clocks(local)
    clk.start()
    st = torch.cuda.current_stream()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    barrier()
    e0.record(st)
    for _ in range(args.steps):
        one_run()
    e1.record(st)
    barrier()
    clocks = clk.stop()
    ms = e0.elapsed_time(e1)
    sim.check()
    ms = max_over_ranks(ms, world, dev)
    value = whole_job_rate(cells * NS * args.steps, world, ms)

    # dominant kernel: time fused passes individually (2 passes of spp steps)
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(10)]
    sim.reset()
    for a, b in ev:
        a.record(st)
        sim.step(2 * spp, steps_per_pass=spp)
        b.record(st)
    torch.cuda.synchronize()
    pass_ms = statistics.median(a.elapsed_time(b) for a, b in ev) / 2
    peak, peak_kind = _peaks()
    algo_bytes = BYTES_PER_CELL_UPDATE * cells * spp
    achieved = algo_bytes / (pass_ms / 1e3) / 1e9
    tb = NCU_TRAFFIC_BYTES_PER_CELL_PASS.get(spp)
    traffic = None if tb is None else tb * cells

    # e2e through the public API with host buffers
    e2e = None
    if not args.no_e2e:
        e2e = run_e2e(sim, args, st, world, dev)

    extra = None
    if rank == 0 and not args.no_extra:
        del sim
        torch.cuda.empty_cache()
        extra = run_secondary(args, st, world)

    cpu = None
    if rank == 0 and world == 1 and not args.no_cpu:
        cpu = cpu_best_rate(NX, NY, int(os.environ.get("FDTD_CPU_SAMPLE_STEPS", "150")))
        cpu["unit"] = UNIT
        cpu["kind"] = "port"
        one = cpu_port_rate(NX, NY, int(os.environ.get("FDTD_CPU_SAMPLE_STEPS_1T", "10")), threads=1,
                            native=cpu["build"] != "gcc -O3 -fopenmp")
        cpu["single_thread"] = {"value": one["value"], "cores": 1, "sample": one["sample"], "build": one["build"]}
        try:
            cpu["numpy_reference_form"] = numpy_reference_rate()
        except Exception as exc:  # reported, never fatal to the bench line
            cpu["numpy_reference_form"] = {"error": f"{type(exc).__name__}: {exc}"}
        from oracle import ccore
        ccore.lib32().oracle_set_threads(cpu["cores"])

    if rank == 0:
        line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
                "warmup": max(args.warmup, 3), "ms_per_step": ms / args.steps, "higher_is_better": True,
                "scaling": "weak", "vs_baseline": None, "dtype": "f32",
                "data": "synthetic (deterministic benchmark program, no RNG)",
                "config": {"workload": WORKLOAD, "grid": [NX, NY], "time_steps_per_bench_step": NS,
                           "steps_per_pass": spp, "parallelism": f"replicas x{world}",
                           "l2": "inputs larger than L2 (3.8 GB of fields per pass)"},
                "hbm_frac_algorithmic": value * BYTES_PER_CELL_UPDATE / peak,
                "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s",
                             "frac": achieved / peak, "traffic": traffic, "peak_kind": peak_kind,
                             "kernel": f"k_march<K={spp}> (one fused pass = {spp} time steps)",
                             "algorithmic_bytes_per_launch": algo_bytes, "launch_ms": pass_ms},
                "e2e": e2e, "cpu_baseline": cpu, "clocks": clocks,
                "gpu_launches": passes_per_run * args.steps, "secondary_workloads": extra}
        print(json.dumps(line), flush=True)
    if world > 1:
        dist.destroy_process_group()


def run_secondary(args, st, world) -> dict:
    """The other workloads of the path, measured after the headline (not part of `value`)."""
    import torch
    out = {"fd1d_dielectric_ke200_1000steps": _bench_fd1d(st)}
    batch = _bench_batch1d(st, cpu=not args.no_cpu)
    out["batch1d_4096_slabs_8000steps"] = batch
    out["fd2d_tfsf_dft_2048sq"] = _bench_tfsf_dft(st)
    out["adjoint_1024sq_3000steps"] = _bench_adjoint(st)
    out["surrogate_fno_batch65536"] = _bench_surrogate(st, batch["spectra_per_s"])
    torch.cuda.empty_cache()
    return out


def _bench_tfsf_dft(st, n: int = 2048, steps: int = 400) -> dict:
    """The fd2d_3_4 program (TF/SF plane wave, lossy cylinder, PML, 3-frequency
    full-field DFT) at n^2 through fdtd2d_step_n: fused passes of 4 steps (the
    incident line advanced ahead in one launch per 64 steps), timed beside
    the same step as three launches (one-step calls) and the nine
    per-function launches of the reference's loop."""
    import torch

    from simulation_gb300 import fd2d as G
    dt = 0.01 / 6e8
    naz, nbz = G.dielectric(n, n, 32, n // 8, dt, 30.0, 0.30)
    sim = G.SimTM2D(n, n, pml=G.pmlparam(n, n, 32), naz=naz, nbz=nbz, lossy=True, tfsf_npml=32,
                    freq=[50e6, 300e6, 700e6], dt=dt, ns=3 * steps + 40)

    def three_launch(k):
        for _ in range(k):
            sim.step(1)

    # the same grid, map and PML without the extras: the plain fused kernel
    plain = G.SimTM2D(n, n, pml=G.pmlparam(n, n, 32), naz=naz, nbz=nbz, lossy=True, dt=dt, ns=3 * steps + 40,
                      source=G.PointSource(n // 2, n // 2, ("gauss", 20, 6.0)))
    out = {}
    for name, fn in (("fused", sim.step), ("three_launch", three_launch), ("per_function", sim.step_per_function),
                     ("plain_fused_no_extras", plain.step)):
        fn(20)
        e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        e0.record(st)
        fn(steps)
        e1.record(st)
        torch.cuda.synchronize()
        out[f"{name}_Gcell_updates_per_s"] = n * n * steps / (e0.elapsed_time(e1) / 1e3) / 1e9
    nf = 3
    # fused pass of K = 4 steps: the 60 field bytes of the lossy PML pass
    # plus the DFT accumulators read and written once (16 bytes per frequency)
    bpc = (60 + 16 * nf) / 4
    out["fused_bytes_per_cell_update"] = bpc
    out["fused_GBps_algorithmic"] = out["fused_Gcell_updates_per_s"] * bpc
    out["grid"] = [n, n]
    out["launches_per_step"] = {"fused": 0.25 + 1 / 64, "three_launch": 3, "per_function": 9}
    del sim, plain
    return out


def _bench_fd1d(st, reps: int = 20) -> dict:
    """Plain 1D dielectric case: ke=200, hard source at k=5, 1000 steps, one fused launch."""
    import torch

    from simulation_gb300 import fd1d as G1
    sim = G1.program("config1", ns=1000)
    for _ in range(5):
        sim.t = 0
        sim.step(1000)
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for _ in range(reps):
        sim.t = 0
        sim.step(1000)
    e1.record(st)
    torch.cuda.synchronize()
    us = e0.elapsed_time(e1) * 1e3 / reps
    # 20 B per cell-update (ex, hy, cb read; ex, hy written) if it were streamed:
    # the line lives in registers, and the run is bound by the step's latency
    res = {"us_per_run": us, "Gcell_updates_per_s": 200 * 1000 / us / 1e3, "kernel_launches_per_run": 1,
           "bytes_per_cell_update": 20, "GBps_algorithmic": 200 * 1000 * 20 / us / 1e3, "bound": "latency"}
    # the same run captured once in a CUDA graph and replayed (no host work per run)
    g = torch.cuda.CUDAGraph()
    cap = torch.cuda.Stream()
    cap.wait_stream(st)
    with torch.cuda.stream(cap):
        with torch.cuda.graph(g, stream=cap):
            sim.t = 0
            sim.step(1000)
    st.wait_stream(cap)
    g.replay()
    torch.cuda.synchronize()
    e0.record(st)
    for _ in range(reps):
        g.replay()
    e1.record(st)
    torch.cuda.synchronize()
    res["us_per_run_graph"] = e0.elapsed_time(e1) * 1e3 / reps
    try:  # the same run through the reference's NumPy form (float64 restatement), one host thread
        from oracle import fd1d as O1
        kw = O1.program("config1")
        O1.run(**kw)
        t0 = time.perf_counter()
        O1.run(**kw)
        el = time.perf_counter() - t0
        res["cpu_baseline"] = {"us_per_run": el * 1e6, "cores": 1, "kind": "port",
                               "sample": "one config-1 run (ke=200, 1000 steps), float64 NumPy form of the reference"}
    except Exception as exc:  # reported, never fatal to the bench line
        res["cpu_baseline"] = {"error": f"{type(exc).__name__}: {exc}"}
    try:  # and through the float32 C port of the reference's fd1d C loop (fd1d/clang/fd1d_1_3.c), one thread
        res["cpu_baseline_c"] = _fd1d_config1_c()
    except Exception as exc:
        res["cpu_baseline_c"] = {"error": f"{type(exc).__name__}: {exc}"}
    return res


def _fd1d_config1_c(budget_s: float = 2.0) -> dict:
    """Config 1 (ke=200, 1000 steps, hard Gaussian source at k=5, ABC) on the
    float32 C port, built for this host's CPU where possible; runs repeat from
    zero fields until about ``budget_s`` seconds have passed."""
    import numpy as np

    from oracle import ccore
    from oracle import fd1d as O1
    lib, build = ccore.lib32_native(), "native"
    if lib is None:
        lib, build = ccore.lib32(), "portable"
    kw = O1.program("config1")
    nx = 200
    cb = np.asarray(kw["cb"], dtype=np.float32)
    table = np.array([O1.gaussian(t, 40, 12.0) for t in range(1, 1001)])
    runs, el = 0, 0.0
    while el < budget_s:
        f = {k: np.zeros(nx, dtype=np.float32) for k in ("ex", "hy")}
        f["bc"] = np.zeros(4, dtype=np.float32)
        t0 = time.perf_counter()
        ccore.fd1d_steps(lib, np.float32, nx, 0, 0, 1000, {"cb": cb}, 1, 5, table, True, f)
        el += time.perf_counter() - t0
        runs += 1
    return {"us_per_run": el / runs * 1e6, "cores": 1, "kind": "port", "build": build, "host": host_cpu(),
            "sample": f"{runs} config-1 runs (ke=200, 1000 steps) on the float32 C port of the reference's fd1d C loop"}


def _bench_batch1d(st, nruns: int = 4096, autotune: bool = True, cpu: bool = False) -> dict:
    """Batched uneven 1D slab runs: ke ~ U[500,20000], 8000 steps, 64-frequency probes."""
    import torch

    from simulation_gb300 import batch1d as B
    batch = B.slab_batch(nruns, seed=0)
    runner = B.BatchRunner(batch, nsteps=8000)
    tuned = B.autotune(runner, probe_steps=400, reps=1) if autotune else {"tuning": runner.tuning}
    runner.run()
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    runner.run()
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    cells = int(batch.ke.sum()) * 8000
    res = {"ms": ms, "Gcell_updates_per_s": cells / ms / 1e6, "spectra_per_s": batch.nruns / ms * 1e3,
           "tuning": tuned["tuning"], "status": int(runner.status.item()),
           "runs_done": int(runner.done.sum().item())}
    # for comparison only: the rate at which a streamed kernel would move the
    # 24 B of a cell-update (ex, hy, ca, cb read; ex, hy written); the state is
    # on chip here, so this exceeds the HBM peak by construction
    peak, kind = _peaks()
    res["hbm_equivalent"] = {"bytes_per_cell_update": 24, "GBps": res["Gcell_updates_per_s"] * 24,
                             "frac_of_peak": res["Gcell_updates_per_s"] * 24 / peak, "peak_kind": kind}
    if cpu:
        res["cpu_baseline"] = _cpu_batch1d(batch, runner)
    return res


def _cpu_batch1d(batch, runner, nsample: int = 64) -> dict:
    """The same runs in the C port of the per-run loop (float32, one run per
    OpenMP thread, all host cores) on a seeded sample of the batch."""
    import numpy as np

    from oracle import ccore
    from simulation_gb300 import batch1d as B
    idx = np.random.default_rng(0).choice(batch.nruns, size=min(nsample, batch.nruns), replace=False)
    b = batch.subset(idx)
    lca, lcb = B.layer_coeffs(b.epsr, b.sigma)
    ns = runner.nsteps
    tab = runner.src_table.double().cpu().numpy()[:ns]
    dc, ds = runner.dft_cos.double().cpu().numpy()[:ns], runner.dft_sin.double().cpu().numpy()[:ns]
    best = None
    # the faster of the portable and the host-tuned builds
    for lib, build in ((ccore.lib32(), "gcc -O3 -fopenmp"), (ccore.lib32_native(), "gcc -O3 -march/-mcpu=native -fopenmp")):
        if lib is None:
            continue
        lib.oracle_set_threads(os.cpu_count() or 1)
        t0 = time.perf_counter()
        ccore.fd1d_batch(lib, np.float32, b.ke, b.layer_off, b.layer_start, b.layer_end, lca, lcb, b.src_k, tab, ns,
                         dc, ds, b.probe_in, b.probe_out)
        el = time.perf_counter() - t0
        if best is None or el < best[0]:
            best = (el, build, int(lib.oracle_threads()))
    el, build, cores = best
    return {"Gcell_updates_per_s": float(b.ke.sum()) * ns / el / 1e9, "spectra_per_s": b.nruns / el,
            "cores": cores, "kind": "port", "build": build,
            "sample": f"{b.nruns} runs of the batch, {ns} steps (float32 C port, OpenMP over runs)"}


def _bench_adjoint(st) -> dict:
    """Gradient of J = sum_t Ez(probe)^2 w.r.t. eps_r on a 256^2 design box of a
    1024^2 lossy PML grid, 3000 steps, checkpoint every 64 steps."""
    import torch

    from simulation_gb300 import adjoint as A
    pr, eps = A.design_problem(seed=0)
    pr.set_eps(eps)
    for _ in range(2):  # eager sweeps, then the CUDA graphs are captured
        pr.forward()
        pr.gradient_eps()
    ev = [torch.cuda.Event(enable_timing=True) for _ in range(3)]
    torch.cuda.synchronize()
    ev[0].record(st)
    pr.forward()
    ev[1].record(st)
    pr.gradient_eps()
    ev[2].record(st)
    torch.cuda.synchronize()
    fwd, rev = ev[0].elapsed_time(ev[1]), ev[1].elapsed_time(ev[2])
    cu = pr.nx * pr.ny * pr.ns
    # algorithmic bytes per cell and time step of this problem (lossless box: no iz, nbz):
    # forward, passes of 2 steps: dz, hx, hy, ihx, ihy, naz in and dz, ez, hx, hy,
    # ihx, ihy out once per pass (48 B / 2); reverse: the recompute pass the same
    # plus the recorded dz, hx, hy of every step (12 B), and the two-step
    # reverse kernel: both states before the steps (2 x 12 B), naz, the 5
    # adjoints in and out once per 2 steps ((24 + 4 + 40) B / 2)
    fwd_b = 48 / 2
    rev_b = 48 / 2 + 12 + (24 + 4 + 40) / 2
    res = {"forward_ms": fwd, "reverse_ms": rev, "forward_Gcell_updates_per_s": cu / fwd / 1e6,
           "reverse_Gcell_updates_per_s": cu / rev / 1e6, "checkpoint": pr.cp, "cuda_graphs": pr.use_graphs,
           "bytes_per_cell_update": {"forward": fwd_b, "reverse": rev_b},
           "GBps_algorithmic": {"forward": cu / fwd / 1e6 * fwd_b, "reverse": cu / rev / 1e6 * rev_b}}
    del pr
    return res


def run_only(args) -> None:
    import torch
    st = torch.cuda.current_stream()
    if args.only == "adjoint":
        res = _bench_adjoint(st)
    elif args.only == "batch1d":
        res = _bench_batch1d(st, nruns=args.batch if args.batch != 65536 else 4096, autotune=False)
    elif args.only == "fd1d":
        res = _bench_fd1d(st, reps=5)
    elif args.only == "tfsf":
        res = _bench_tfsf_dft(st)
    else:
        fdtd = _bench_batch1d(st, cpu=False)["spectra_per_s"]  # the denominator: batched FDTD, 4096 runs
        res = _bench_surrogate(st, fdtd, n=args.batch)
    print(json.dumps({"workload": args.only, **res}), flush=True)


def _bench_surrogate(st, fdtd_spectra_per_s: float | None, n: int = 65536) -> dict:
    """The learned surrogate, trained here and served through its FDTD judge.

    * training: FDTD_SURR_TRAIN profiles (default 200k) of the batched-slab
      distribution solved by the batched kernel, FDTD_SURR_SAMPLES minibatch
      samples (default 2M) of Adam through the library's own forward and
      backward kernels (all timed and reported);
    * one served request of n = 65536 held-out profiles (another seed): inputs
      built on the device, network + frame, 1% re-solved by batched FDTD on a
      second stream, replaced where off by more than 1%.  Its spectra/s is the
      judged throughput; every one of its spectra is then solved by FDTD
      (outside the timed region) to report the served output's error:
      median, p90, fraction within 1% and the relative L2 of the whole set;
    * the network alone (no judge) at the same batch, its tensor-core FLOPs
      against the measured dense BF16 peak."""
    import numpy as np
    import torch

    from simulation_gb300 import batch1d as B1
    from simulation_gb300 import surrogate as S
    ntrain = int(os.environ.get("FDTD_SURR_TRAIN", "200000"))
    samples = int(os.environ.get("FDTD_SURR_SAMPLES", "2000000"))
    ev = lambda: torch.cuda.Event(enable_timing=True)  # noqa: E731
    e0, e1 = ev(), ev()
    e0.record(st)
    X, Y, _ = S.generate_dataset(ntrain, seed=100, on_device=True)
    e1.record(st)
    torch.cuda.synchronize()
    data_s = e0.elapsed_time(e1) / 1e3
    m = S.FNO(seed=0)
    e0.record(st)
    hist = S.train(m, X, Y, samples=samples, lr=1e-3, lr_final=1e-5, log_every=1000)
    e1.record(st)
    torch.cuda.synchronize()
    train_s = e0.elapsed_time(e1) / 1e3
    del X, Y
    torch.cuda.empty_cache()
    req = B1.slab_batch(n, seed=777)
    served = S.time_served(m, req, check_frac=0.01, tol=0.01, reps=1)
    pred = served.pop("pred")
    ref = torch.empty_like(pred)
    for s in range(0, n, 4096):
        ref[s:s + 4096] = S.solve_fdtd_device(req.subset(np.arange(s, min(n, s + 4096))))
    err = S.rel_l2_spectrum_device(pred, ref).cpu().numpy()
    net_err = S.rel_l2_spectrum_device(m.spectrum(S.device_features(req)), ref).cpu().numpy()
    agg = float(torch.linalg.vector_norm((pred - ref).double()) / torch.linalg.vector_norm(ref.double()))
    sps_net = S.time_inference(m, n=n, chunk=4096, reps=1)
    fl = S.flops_per_sample(m)
    peak = _peaks_bf16()
    vs = (lambda v: None if not fdtd_spectra_per_s else v / fdtd_spectra_per_s)
    res = {"request": n, "judged_spectra_per_s": served["spectra_per_s"],
           "judged_vs_batched_fdtd": vs(served["spectra_per_s"]),
           "checked": served["checked"], "fell_back": served["fell_back"],
           "served_error": {"median": float(np.median(err)), "p90": float(np.quantile(err, 0.9)),
                            "frac_le_1pct": float(np.mean(err <= 0.01)), "relL2_of_set": agg},
           "network_only_error": {"median": float(np.median(net_err)), "frac_le_1pct": float(np.mean(net_err <= 0.01))},
           "spectra_per_s": sps_net, "vs_batched_fdtd_spectra_per_s": vs(sps_net),
           "gflop_per_sample": fl / 1e9, "tflops": sps_net * fl / 1e12,
           "frac_of_bf16_peak": None if peak is None else sps_net * fl / 1e12 / peak,
           "training": {"profiles": ntrain, "samples_seen": samples, "dataset_s": data_s, "train_s": train_s,
                        "loss_first_last": [hist[0][1], hist[-1][1]]},
           "batched_fdtd_spectra_per_s": fdtd_spectra_per_s}
    del m
    torch.cuda.empty_cache()
    return res


def host_link_gbps(host_src, dev_buf, host_dst, reps: int = 3) -> dict:
    """Pinned host <-> device copy rate (GB/s) of one field array, each
    direction alone, best of ``reps``: what the pipeline fill (the first
    request's upload) and drain (the last one's download) run at."""
    import torch
    st = torch.cuda.current_stream()
    out = {}
    for name, dst, src in (("h2d", dev_buf, host_src), ("d2h", host_dst, dev_buf)):
        best = None
        for _ in range(reps):
            e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            e0.record(st)
            dst.copy_(src, non_blocking=True)
            e1.record(st)
            torch.cuda.synchronize()
            ms = e0.elapsed_time(e1)
            best = ms if best is None else min(best, ms)
        out[name] = src.numel() * 4 / (best / 1e3) / 1e9 if best else None
    return out


def run_e2e(sim, args, st, world, dev) -> dict:
    """Same runs through SimTM2D with host (pinned) buffers copied in and out.

    Two simulations alternate, as a server handling a stream of requests would
    run them: while one computes, the other's results and next inputs cross
    the host link on the copy engines.  Each simulation has an upload, a
    compute and a download stream; an array's upload waits only for the
    download of the same array, so the two directions of the link overlap.
    The kernels of the two simulations never overlap (each step's compute
    waits for the previous step's), so the GPU work per step is that of
    ``value``; every step still copies all of its inputs in and all of its
    results out.  The first upload and the last download cannot overlap any
    compute (pipeline fill and drain, 25 ms to 300 ms depending on the host
    link), so the e2e run takes at least E2E_MIN_STEPS steps."""
    import torch

    from simulation_gb300 import fd2d as G
    keys_in = ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy", "naz", "nbz")
    keys_out = ("dz", "ez", "iz", "hx", "hy", "ihx", "ihy")
    host_in = {k: torch.zeros((NX, NY), dtype=torch.float32, pin_memory=True) for k in keys_in}
    host_in["naz"].copy_(sim.naz.cpu())
    host_in["nbz"].copy_(sim.nbz.cpu())
    pml_host = {k: getattr(sim.pml, k).cpu().pin_memory() for k in sim.pml._fields}
    sims = [sim, G.benchmark_sim(NX, NY, NPML, GRADE, RGRID, EPSR, SIGMA, ns=NS, device=dev,
                                 steps_per_pass=args.spp)]
    up = [torch.cuda.Stream(device=dev) for _ in sims]
    comp = [torch.cuda.Stream(device=dev) for _ in sims]
    down = [torch.cuda.Stream(device=dev) for _ in sims]
    host_out = [{k: torch.empty((NX, NY), dtype=torch.float32, pin_memory=True) for k in keys_out} for _ in sims]
    out_done = [{} for _ in sims]  # array -> event: its last download finished reading the device buffer
    last_compute = [None for _ in sims]  # this simulation's previous compute (it reads every input)
    # inputs that are not downloaded go first, while the other arrays are still on their way out
    order_in = [k for k in keys_in if k not in keys_out] + [k for k in keys_in if k in keys_out]

    def one(k, prev_done):
        i = k % 2
        s, o = sims[i], host_out[i]
        with torch.cuda.stream(up[i]):
            if last_compute[i] is not None:
                up[i].wait_event(last_compute[i])
            u0 = torch.cuda.Event(enable_timing=True)
            u0.record(up[i])
            for key in order_in:
                ev = out_done[i].get(key)
                if ev is not None:
                    up[i].wait_event(ev)
                getattr(s, key).copy_(host_in[key], non_blocking=True)
            for key, v in pml_host.items():
                getattr(s.pml, key).copy_(v, non_blocking=True)
            inputs = torch.cuda.Event(enable_timing=True)
            inputs.record(up[i])
            uploads.append((u0, inputs))
        with torch.cuda.stream(comp[i]):
            comp[i].wait_event(inputs)
            if prev_done is not None:
                comp[i].wait_event(prev_done)  # compute after the previous step's compute
            begin = torch.cuda.Event(enable_timing=True)
            begin.record(comp[i])
            s.t = 0
            s.step(NS)
            done = torch.cuda.Event(enable_timing=True)
            done.record(comp[i])
            last_compute[i] = done
            spans.append((begin, done))
        with torch.cuda.stream(down[i]):
            down[i].wait_event(done)
            d0 = torch.cuda.Event(enable_timing=True)
            d0.record(down[i])
            for key in keys_out:
                o[key].copy_(getattr(s, key), non_blocking=True)
                ev = torch.cuda.Event(enable_timing=True)
                ev.record(down[i])
                out_done[i][key] = ev
            downloads.append((d0, ev))
        return done

    spans = []  # (begin, end) events of each step's compute
    uploads, downloads = [], []  # (begin, end) events of each step's copies
    link = host_link_gbps(host_in["dz"], sims[0].dz, host_out[0]["dz"])
    # warm-up requests, the last thing before the timed region: workspaces,
    # tables, and every host buffer of both simulations recently copied
    done = None
    for k in range(2):
        done = one(k, done)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record(st)
    for x in up + comp + down:
        x.wait_stream(st)
    done = None
    steps = max(args.steps, E2E_MIN_STEPS)
    spans.clear()
    uploads.clear()
    downloads.clear()
    for k in range(steps):
        done = one(k, done)
    for x in up + comp + down:
        st.wait_stream(x)
    e1.record(st)
    torch.cuda.synchronize()
    ms = e0.elapsed_time(e1)
    compute_each = [b.elapsed_time(d) for b, d in spans]
    compute_ms = statistics.median(compute_each)
    # the gaps between one request's compute and the next (pipeline stalls),
    # and the time before the first compute (fill) and after the last (drain)
    gaps = [spans[k - 1][1].elapsed_time(spans[k][0]) for k in range(1, len(spans))]
    lead, tail = e0.elapsed_time(spans[0][0]), spans[-1][1].elapsed_time(e1)
    for s in sims:
        s.check()
    h2d = sum(v.numel() * 4 for v in host_in.values()) + sum(v.numel() * 4 for v in pml_host.values())
    d2h = sum(v.numel() * 4 for v in host_out[0].values())
    del sims[1]
    ms = max_over_ranks(ms, world, dev)
    return {"value": whole_job_rate(NX * NY * NS * steps, world, ms), "unit": UNIT,
            "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h, "ms_per_step": ms / steps, "steps": steps,
            "simulations_in_flight": 2, "copy_streams": "upload and download per simulation",
            "host_link_GBps": link, "compute_ms_per_step_median": compute_ms,
            "compute_ms_each": [round(x, 2) for x in compute_each], "gap_ms_each": [round(x, 2) for x in gaps],
            "fill_ms": lead, "drain_ms": tail,
            "upload_ms_each": [round(a.elapsed_time(b), 2) for a, b in uploads],
            "download_ms_each": [round(a.elapsed_time(b), 2) for a, b in downloads],
            "fill_drain_ms": (h2d / link["h2d"] + d2h / link["d2h"]) / 1e6 if link["h2d"] and link["d2h"] else None}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=3)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="ours", choices=["ours", "reference"])
    ap.add_argument("--spp", type=int, default=4, help="time steps per fused pass (1..4)")
    ap.add_argument("--grid", type=int, default=8192, help="grid edge (profiling runs use a smaller case)")
    ap.add_argument("--ns", type=int, default=2000, help="time steps per bench step")
    ap.add_argument("--no-e2e", action="store_true")
    ap.add_argument("--no-cpu", action="store_true")
    ap.add_argument("--no-extra", action="store_true", help="skip the secondary workloads")
    ap.add_argument("--only", choices=["surrogate", "adjoint", "batch1d", "fd1d", "tfsf"],
                    help="run one secondary workload alone and print its JSON (profiling runs)")
    ap.add_argument("--batch", type=int, default=65536,
                    help="surrogate spectra per timed pass (--only surrogate); runs for --only batch1d (default 4096)")
    args = ap.parse_args()
    if args.only:
        run_only(args)
        return
    global NX, NY, NS
    NX = NY = args.grid
    NS = args.ns
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
