"""Throughput benchmark of the Cahn–Hilliard time-step hot path on one GB300.

    python bench.py [--gpus N] [--steps K] [--warmup W] [--impl chgb|reference] [--workload NAME]

Metric: cell-steps/s (FP64).  One bench "step" is one output interval of the
reference's driver loop (INTERVAL time steps between two syncs), so that the
end-to-end leg is meaningful: every e2e step uploads the field from pinned
host memory, advances INTERVAL time steps and downloads the field, all
through the C ABI (chgb_upload / chgb_step / chgb_download).

The headline workload is the 3D half of the configuration the reference's
metric is quoted on: 3D Landau `euler`, N=256 (16.7 M cells, 128 MiB per
field, larger than L2), dt=0.005, k=1, M=1, eps=0.9, psi0 = U(-0.01, 0.01)
from a seed.  The other workloads of that configuration (2D pseudospectral
N=1024, and 2D euler N=1024 of the stated target) are reported in
`workloads` with their own roofline.

`--impl reference` times the reference's CPU algorithm (the oracle
restatement of it, C, one box per host thread) on a bounded sample of the
same workload.  Under torchrun only rank 0 runs it.
"""
from __future__ import annotations

import argparse
import ctypes
import json
import os
import statistics
import subprocess
import sys
import threading
import time
from pathlib import Path

import numpy as np

REPO = Path(__file__).resolve().parent
sys.path.insert(0, str(REPO / "cahn-hilliard_gb300"))

INTERVAL = 100          # time steps per bench step (one output interval)
FLUSH_BYTES = 256 << 20  # L2 flush buffer (L2 is 129 MB)

# Algorithmic work per cell-step:
#   bytes_per_cell  the compulsory FP64 state read + write (16 B);
#   fp64_per_cell   instructions of the FP64 pipe per cell and time step for
#                   each kernel variant (1 fused, 2 split, 3 two steps per
#                   launch, 4 cluster-resident, 5 split in block fixed point),
#                   halo recomputation included:
#                   ncu's sm__inst_executed_pipe_fp64 x 32 per cell (the
#                   explicit steps' neighbour sums run on the integer pipe, so
#                   the int64 -> double conversion of each sum is the one FP64
#                   instruction they keep);
#   alu_per_cell    integer-ALU pipe instructions per cell and time step (ncu's
#                   sm__inst_executed_pipe_alu x 32 per cell), where the
#                   neighbour sums made that pipe a binding one;
#   ncu_traffic     dram__bytes_read.sum + dram__bytes_write.sum per time step
#                   from one ncu capture, per variant (profiles/).
WORKLOADS = {
    "euler3d_N256": dict(dims=3, N=256, integrator="euler", dt=0.005, bytes_per_cell=16.0,
                         fp64_per_cell={1: 7.31, 2: 6.0, 5: 2.0 + 1.5}, alu_per_cell={2: 173.8, 5: 69.3 + 55.4},
                         ncu_traffic={2: 135.3e6 + 94.9e6 + 269.6e6 + 115.9e6,
                                      5: 135.4e6 + 94.7e6 + 274.4e6 + 107.1e6},
                         desc="3D Landau euler N=256, dt=0.005, k=1, M=1, eps=0.9, psi0=U(-0.01,0.01)"),
    "euler2d_N1024": dict(dims=2, N=1024, integrator="euler", dt=0.01, bytes_per_cell=16.0,
                          fp64_per_cell={1: 4 * (34 * 34) / (32 * 32) + 2, 2: 5.0, 5: 4.25},
                          alu_per_cell={2: 177.6, 5: 114.6},
                          ncu_traffic={2: 8.39e6 + 16.78e6, 5: 8.41e6},
                          desc="2D Landau euler N=1024, dt=0.01, k=1, M=1, eps=0.9, psi0=U(-0.01,0.01)"),
    "pseudospectral2d_N1024": dict(dims=2, N=1024, integrator="pseudospectral", dt=0.05, bytes_per_cell=16.0,
                                   # fixed-point transforms: FP64 only in f' and the mode update
                                   fp64_per_cell={1: 5.9, 2: 5.9}, alu_per_cell={1: 637.0, 2: 637.0},
                                   ncu_traffic={1: 8.50e6 + 25.34e6, 2: 8.50e6 + 25.34e6},
                                   desc="2D Landau pseudospectral N=1024, dt=0.05, k=1, M=1, eps=0.9, "
                                        "psi0=U(-0.01,0.01)"),
}
WORKLOADS["euler2d_N64"] = dict(
    dims=2, N=64, integrator="euler", dt=0.01, bytes_per_cell=16.0,
    fp64_per_cell={1: (4 * 18 * 18 + 2 * 16 * 16) / (16 * 16), 2: 5.0,
                   3: (4 * (22 * 22 + 18 * 18) + 2 * (20 * 20 + 16 * 16)) / (2 * 16 * 16),
                   4: (4 * 18 * 18 + 2 * 16 * 16) / (16 * 16)}, ncu_traffic={},
    desc="2D Landau euler N=64 (4096 cells), dt=0.01, k=1, M=1, eps=0.9, psi0=U(-0.01,0.01): the reference's "
         "CPU-runnable case, launch-latency bound on one box (many such boxes belong in the batch)")
WORKLOADS["wertheim3d_N128"] = dict(
    dims=3, N=128, integrator="euler_mobility", model="simple_wertheim", dt=1e-4, rho_mean=1.107e-5,
    bytes_per_cell=16.0, fp64_per_cell={2: 51.25 + 16.25}, alu_per_cell={2: 134.6 + 81.4}, ncu_traffic={},
    desc="3D simple_wertheim euler_mobility N=128, free-energy mobility M0 rho X^4, dt=1e-4, dx=10, k=1e6, "
         "rho0=1.107e-5 (about half the sites bonded) with 1% relative noise")
HEADLINE = "euler3d_N256"
SEED = 20240327


_FP64_PEAK = None


def fp64_peak() -> dict | None:
    """Sustained FP64 instruction rate measured live by lib/chgb_fp64_peak."""
    global _FP64_PEAK
    if _FP64_PEAK is None:
        exe = REPO / "cahn-hilliard_gb300" / "lib" / "chgb_fp64_peak"
        try:
            r = subprocess.run([str(exe)], capture_output=True, text=True, timeout=120, check=True)
            _FP64_PEAK = json.loads(r.stdout.strip().splitlines()[-1])
        except Exception as e:  # reported, not fatal
            _FP64_PEAK = {"error": str(e)}
    return _FP64_PEAK


def measured_peaks() -> dict:
    p = REPO / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return {"hbm_gbs": d.get("hbm_gbs"), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons sampled during the timed region."""
    FIELDS = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.hw_slowdown,"
              "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
              "clocks_event_reasons.sw_power_cap")

    def __init__(self, index: int = 0):
        self.index = index
        self.proc = None
        self.lines: list[str] = []

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.index}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.t = threading.Thread(target=self._read, daemon=True)
            self.t.start()
        except Exception:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def __exit__(self, *exc):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except Exception:
                self.proc.kill()

    def summary(self) -> dict:
        sm, mx, reasons = [], None, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [x.strip() for x in ln.split(",")]
            if len(parts) < 7:
                continue
            try:
                sm.append(float(parts[0]))
                mx = float(parts[1])
            except ValueError:
                continue
            for nm, v in zip(names, parts[3:7]):
                if v.lower().startswith("active"):
                    reasons.add(nm)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": mx, "reasons": sorted(reasons),
                "samples": len(sm)}


KERNEL_VARIANT = 0       # 0: picked by timing at create; 1 fused; 2 split; 3 two per launch; 4 cluster;
                         # 5 split in block fixed point (--kernel-variant)


def make_params(w: dict):
    from chgb import config
    if w.get("model") == "simple_wertheim":
        # examples/wertheim/simple.toml's constants (dx = 10, k = 1e6, valence 4, B2 = 2190, Delta from
        # T = 300 K, deltaH = -42200, deltaS = -119.1, salt 0.5, 6 sticky bases); M = M0 rho X^4
        p = config.params(w["dims"], w["N"], w["integrator"], "simple_wertheim", dt=w["dt"], dx=10.0, k=1e6,
                          M=1.0, mobility="free_energy", valence=4, B2=2190.0, delta=config.delta_value(
                              {"T": 300, "deltaH": -42200, "deltaS": -119.1, "salt": 0.5, "sticky_size": 6}, "d"))
    else:
        p = config.params(w["dims"], w["N"], w["integrator"], "landau", dt=w["dt"], k=1.0, M=1.0, epsilon=0.9)
    if w["integrator"] not in ("pseudospectral", "pseudospectral_mobility"):
        p.kernel_variant = KERNEL_VARIANT
    return p


# ---- ranks (replicas only: each rank steps its own box; no collective on the data path)

def dist_ready() -> bool:
    try:
        import torch.distributed as dist
    except ImportError:
        return False
    return dist.is_available() and dist.is_initialized()


def rank_barrier() -> None:
    """Barrier across the ranks of the job (a no-op in a single process)."""
    if dist_ready():
        import torch.distributed as dist
        dist.barrier()


def max_over_ranks(x: float, device: str = "cpu") -> float:
    """The largest of every rank's `x` (the job ends when its slowest rank does)."""
    if not dist_ready():
        return float(x)
    import torch
    import torch.distributed as dist
    t = torch.tensor([float(x)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank: float, world: int, max_seconds: float) -> float:
    """Units all ranks processed divided by the slowest rank's time."""
    return units_per_rank * world / max_seconds


def world_size() -> int:
    return int(os.environ.get("WORLD_SIZE", "1"))


def initial_field(w: dict) -> np.ndarray:
    from chgb import config
    return config.init_density(w["dims"], w["N"], [w.get("rho_mean", 0.0)], initial_A=1e-2, seed=SEED)


def workload_config(name: str) -> dict:
    """The `config` of a workload's JSON line, the same for both arms."""
    w = WORKLOADS[name]
    cells = w["N"] ** w["dims"]
    big = cells * 8 * 2 > 160e6
    return {"workload": w["desc"], "cells": cells, "time_steps_per_bench_step": INTERVAL,
            "l2": "inputs larger than L2" if big else "L2 flushed between bench steps"}


def bench_gpu(name: str, steps: int, warmup: int, with_e2e: bool, ranks: bool = True) -> dict:
    """One workload on this rank's GPU.  ranks=True brackets the timed regions
    with barriers across the job's ranks (every rank must call it); the extra
    workloads rank 0 measures alone pass False."""
    import torch
    from chgb import abi
    from chgb.sim import CahnHilliard

    w = WORKLOADS[name]
    lib = abi.load_library()
    p = make_params(w)
    cells = p.bins
    rho0 = initial_field(w)
    stream = torch.cuda.Stream()
    sim = CahnHilliard(p, rho0, lib=lib)
    sim.set_stream(stream.cuda_stream)
    flush = torch.empty(FLUSH_BYTES // 4, dtype=torch.float32, device="cuda")
    big = cells * 8 * 2 > 160e6

    # ---- device-resident throughput -------------------------------------
    for _ in range(warmup):
        sim.evolve(INTERVAL)
    sim.synchronize()
    torch.cuda.synchronize()
    starts = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    ends = [torch.cuda.Event(enable_timing=True) for _ in range(steps)]
    l0 = sim.launches
    with ClockSampler() as clk:
        torch.cuda.synchronize()
        if ranks:
            rank_barrier()
        for i in range(steps):
            if not big:
                with torch.cuda.stream(stream):
                    flush.add_(1.0)
            with torch.cuda.stream(stream):
                starts[i].record(stream)
            sim.evolve(INTERVAL)
            with torch.cuda.stream(stream):
                ends[i].record(stream)
        torch.cuda.synchronize()
        if ranks:
            rank_barrier()
    step_ms = [s.elapsed_time(e) for s, e in zip(starts, ends)]
    launches = sim.launches - l0
    variant = sim.kernel_variant
    t_total = sum(step_ms) / 1e3
    value = cells * INTERVAL * steps / t_total
    # one time step = one launch (fused / pseudospectral 1D) or 2-4 launches;
    # the roofline is taken per time step, the unit the algorithmic bytes count
    tstep_s = t_total / (INTERVAL * steps)
    peaks = measured_peaks()
    achieved = w["bytes_per_cell"] * cells / tstep_s / 1e9
    out = {
        "value": value,
        "ms_per_step": sum(step_ms) / steps,
        "gpu_launches": launches,
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "traffic": None, "peak_source": peaks["source"],
                     "bytes_per_time_step": w["bytes_per_cell"] * cells, "time_step_ms": tstep_s * 1e3,
                     "launches_per_time_step": launches / (INTERVAL * steps), "kernel_variant": variant,
                     "binding_resource": "fp64 and integer-ALU pipes (fp64_roofline, alu_roofline): GB300 "
                                         "runs FP64 at 1/64 of FP32, so an FP64 stencil issues at the FP64 "
                                         "ceiling long before HBM; the neighbour sums run on the integer ALU"},
        "clocks": clk.summary(),
        "config": workload_config(name),
    }
    traffic = (w.get("ncu_traffic") or {}).get(variant)
    if traffic:
        out["roofline"]["traffic"] = traffic
    fp64_count = (w.get("fp64_per_cell") or {}).get(variant)
    if fp64_count:
        pk = fp64_peak()
        achieved_gi = fp64_count * cells / tstep_s / 1e9
        peak_gi = pk.get("dfma_ginst_s") if pk else None
        out["fp64_roofline"] = {"bound": "fp64", "achieved": achieved_gi, "peak": peak_gi,
                                "unit": "G FP64 inst/s", "frac": achieved_gi / peak_gi if peak_gi else None,
                                "fp64_inst_per_cell": fp64_count,
                                "peak_source": "lib/chgb_fp64_peak (DFMA chains, measured in this run)"}
    alu_count = (w.get("alu_per_cell") or {}).get(variant)
    if alu_count:
        # nominal: 16 lanes per clock per SM sub-partition (the peak ncu's
        # sm__pipe_alu_cycles_active percentages refer to) at the SM clock seen
        sm_mhz = (out["clocks"] or {}).get("sm_mhz") or 2070.0
        peak_ti = 152 * 64 * sm_mhz * 1e6 / 1e12
        achieved_ti = alu_count * cells / tstep_s / 1e12
        out["alu_roofline"] = {"bound": "int alu", "achieved": achieved_ti, "peak": peak_ti, "unit": "T ALU inst/s",
                               "frac": achieved_ti / peak_ti, "alu_inst_per_cell": alu_count,
                               "peak_source": "nominal, 64 lanes/clk/SM x 152 SMs at the sampled SM clock"}

    # ---- end to end through the C ABI with pinned host buffers ------------
    if with_e2e:
        h_in = torch.from_numpy(rho0).pin_memory()
        h_out = torch.empty_like(h_in).pin_memory()
        D = ctypes.POINTER(ctypes.c_double)
        pin = ctypes.cast(h_in.data_ptr(), D)
        pout = ctypes.cast(h_out.data_ptr(), D)
        h = sim._h
        for _ in range(max(1, warmup // 2)):
            abi.check(lib, lib.chgb_upload(h, pin, None), h)
            abi.check(lib, lib.chgb_step(h, INTERVAL), h)
            abi.check(lib, lib.chgb_download(h, pout, None), h)
        e_steps = max(2, steps // 2)
        torch.cuda.synchronize()
        if ranks:
            rank_barrier()
        t0 = time.perf_counter()
        for _ in range(e_steps):
            abi.check(lib, lib.chgb_upload(h, pin, None), h)
            abi.check(lib, lib.chgb_step(h, INTERVAL), h)
            abi.check(lib, lib.chgb_download(h, pout, None), h)
        t1 = time.perf_counter()
        if ranks:
            rank_barrier()
        nbytes = cells * 8
        e_max = max_over_ranks(t1 - t0, "cuda") if ranks else t1 - t0
        n_ranks = world_size() if ranks else 1
        out["e2e"] = {"value": whole_job_rate(cells * INTERVAL * e_steps, n_ranks, e_max), "unit": "cell-steps/s",
                      "h2d_bytes_per_step": nbytes, "d2h_bytes_per_step": nbytes,
                      "api": "chgb_upload + chgb_step + chgb_download (C ABI, pinned host buffers)"}
    sim.close()
    return out


# ---------------------------------------------------------------------------
# CPU: the reference's algorithm (oracle restatement), one box per host thread
# ---------------------------------------------------------------------------
def bench_cpu(name: str, seconds_target: float = 12.0, threads: int | None = None) -> dict:
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    from concurrent.futures import ThreadPoolExecutor

    w = WORKLOADS[name]
    p = make_params(w)
    rho0 = initial_field(w)
    threads = threads or os.cpu_count() or 1
    # probe one step on one thread to size the sample
    s = oracle.OracleSim(p, rho0)
    t0 = time.perf_counter()
    s.step(1)
    one = time.perf_counter() - t0
    nsteps = max(1, int(seconds_target / max(one, 1e-6)))
    sims = [oracle.OracleSim(p, rho0) for _ in range(threads)]

    def run(sim):
        sim.step(nsteps)   # ctypes releases the GIL

    t0 = time.perf_counter()
    with ThreadPoolExecutor(max_workers=threads) as ex:
        list(ex.map(run, sims))
    dt = time.perf_counter() - t0
    for sm in sims:
        sm.close()
    value = p.bins * nsteps * threads / dt
    return {"value": value, "unit": "cell-steps/s", "cores": threads, "kind": "port",
            "sample": f"{nsteps} time steps of the full {w['desc']} field on each of {threads} host threads "
                      f"(one independent box per thread), {dt:.1f} s wall"}


BATCH_DESC = ("256 independent 2D Landau replicas, N uniform in {64,128,256,512}, eps~U[0.5,1], "
              "psi0~U[-0.4,0.4]+U(-0.01,0.01), distinct seeds; half euler (dt=0.01, k~U[0.5,1.4]: k above "
              "~1.44 is linearly unstable at this dt) and half pseudospectral (dt=0.05, k~U[0.5,2])")


def batch_replicas(n: int = 256, seed: int = 7):
    from chgb import config
    rng = np.random.default_rng(seed)
    reps, fields = [], []
    for i in range(n):
        N = int(rng.choice([64, 128, 256, 512]))
        eps = float(rng.uniform(0.5, 1.0))
        if i % 2 == 0:
            p = config.params(2, N, "euler", "landau", dt=0.01, k=float(rng.uniform(0.5, 1.4)), epsilon=eps)
        else:
            p = config.params(2, N, "pseudospectral", "landau", dt=0.05, k=float(rng.uniform(0.5, 2.0)), epsilon=eps)
        rho = config.init_density(2, N, [0.0], initial_A=1e-2, seed=1000 + i) + float(rng.uniform(-0.4, 0.4))
        reps.append(p)
        fields.append(rho)
    return reps, fields


def bench_batch(steps: int) -> dict:
    """Batched mode vs looping the plain single-box path over the same replicas."""
    import torch
    from chgb.sim import Batch, CahnHilliard
    reps, fields = batch_replicas()
    cells = sum(p.bins for p in reps)
    # looped plain path: each replica stepped to completion, one after the other
    sims = [CahnHilliard(p, f) for p, f in zip(reps, fields)]
    for s in sims:
        s.evolve(2)
        s.synchronize()
    torch.cuda.synchronize()
    t0 = time.perf_counter()
    for s in sims:
        s.evolve(steps)
        s.synchronize()
    t_loop = time.perf_counter() - t0
    loop_launches = sum(s.launches for s in sims)
    for s in sims:
        s.close()
    # batched
    b = Batch(reps)
    for i, f in enumerate(fields):
        b.upload(i, f)
    b.step(2)
    b.synchronize()
    l0 = b.launches
    t0 = time.perf_counter()
    b.step(steps)
    b.synchronize()
    t_batch = time.perf_counter() - t0
    launches = b.launches - l0
    tile = b.euler_tile
    b.close()
    return {"value": cells * steps / t_batch, "unit": "cell-steps/s", "loop_value": cells * steps / t_loop,
            "batch_speedup": t_loop / t_batch, "gpu_launches": launches,
            "loop_gpu_launches": loop_launches, "euler_tile": tile,
            "config": {"workload": BATCH_DESC, "replicas": len(reps), "cells": cells,
                       "time_steps_timed": steps, "time_steps_in_configuration": 2000,
                       "timing": "host wall clock around step + synchronize, both legs"}}


def bench_adjoint(integrator: str, steps: int = 2000, every: int = 45) -> dict:
    """Cost of one adjoint step (recompute + adjoint) relative to one forward
    step, on the adjoint configuration: 2D Landau N=256, T steps, a checkpoint
    every 45 steps, loss sum_q (S - S*)^2."""
    from chgb import config
    from chgb.sim import Adjoint, CahnHilliard
    N = 256
    dt = 0.01 if integrator == "euler" else 0.05
    p = config.params(2, N, integrator, "landau", dt=dt, k=1.0, M=0.9, epsilon=0.9)
    rho0 = config.init_density(2, N, [0.0], initial_A=0.02, seed=17)
    sim = CahnHilliard(p, rho0)
    sim.evolve(50)
    sim.synchronize()
    t0 = time.perf_counter()
    sim.evolve(steps)
    sim.synchronize()
    t_fwd = time.perf_counter() - t0
    sim.close()
    adj = Adjoint(p, steps, every)
    adj.forward(rho0)                       # warm-up of both passes
    sq, _ = adj.forward(rho0)
    adj.backward(dl_dsq=np.ones_like(sq))
    t0 = time.perf_counter()
    sq, _ = adj.forward(rho0)
    t1 = time.perf_counter()
    adj.backward(dl_dsq=2.0 * sq)
    t2 = time.perf_counter()
    adj.close()
    return {"forward_ms_per_step": 1e3 * t_fwd / steps,
            "checkpointed_forward_ms_per_step": 1e3 * (t1 - t0) / steps,
            "backward_ms_per_step": 1e3 * (t2 - t1) / steps,
            "adjoint_step_cost_vs_forward": (t2 - t1) / t_fwd,
            "gradient_cost_vs_forward": (t2 - t0) / t_fwd,
            "config": {"workload": f"2D Landau {integrator} N={N}, T={steps}, checkpoint every {every}; loss "
                                   "sum_q (S(q) - S*(q))^2; backward = segment recompute + adjoint step",
                       "timing": "host wall clock around synchronised calls"}}


def _oracle():
    sys.path.insert(0, str(REPO / "oracle"))
    import oracle
    return oracle


def _gpu_rate(sim, steps: int) -> tuple[float, int]:
    """(seconds, launches) of `steps` steps, synchronised on both sides."""
    sim.synchronize()
    l0 = sim.launches
    t0 = time.perf_counter()
    sim.evolve(steps)
    sim.synchronize()
    return time.perf_counter() - t0, sim.launches - l0


def bench_psmob(steps: int = 200) -> dict:
    """`pseudospectral_mobility` with the gel mobility: the M0-splitting path
    on 2D Landau N=1024 and the GMRES path on N=256, against the oracle's CPU
    restatement on one host thread (a few steps of the same fields)."""
    from chgb import abi, config
    from chgb.sim import CahnHilliard
    oracle = _oracle()

    def gel(p):
        p.mobility_type = abi.MOBILITIES["gel"]
        p.gel_phi_critical, p.gel_c0, p.gel_M_c = 0.3, 0.1, 20.0
        p.gel_beta_delta_F = 10.0 / (1.0 - 0.9) - np.log(24000.0)
        return p

    out = {}
    for name, N, gmres, nsteps, cpu_steps in (("m0_splitting_2d_N1024", 1024, False, steps, 2),
                                              ("gmres_2d_N256", 256, True, max(10, steps // 10), 2)):
        p = gel(config.params(2, N, "pseudospectral_mobility", "landau", dt=0.02, k=1.0, epsilon=0.9, S=0.3))
        if gmres:
            p.use_gmres, p.gmres_restart, p.gmres_max_iter, p.gmres_tol = 1, 10, 200, 1e-11
        rho0 = config.init_density(2, N, [-0.1], initial_A=0.3, seed=3)
        sim = CahnHilliard(p, rho0)
        sim.evolve(5)
        dt_gpu, launches = _gpu_rate(sim, nsteps)
        sim.close()
        ref = oracle.OracleSim(p, rho0)
        t0 = time.perf_counter()
        ref.step(cpu_steps)
        dt_cpu = time.perf_counter() - t0
        ref.close()
        out[name] = {"value": N * N * nsteps / dt_gpu, "unit": "cell-steps/s", "ms_per_step": 1e3 * dt_gpu / nsteps,
                     "launches_per_step": launches / nsteps,
                     "cpu_baseline": {"value": N * N * cpu_steps / dt_cpu, "unit": "cell-steps/s", "cores": 1,
                                      "kind": "port", "sample": f"{cpu_steps} steps of the same field"}}
    out["config"] = {"workload": "pseudospectral_mobility, 2D Landau (eps=0.9, k=1), gel mobility (phi_c=0.3, c0=0.1, "
                                 "M_c=20), S=0.3, dt=0.02, rho0=-0.1 with A=0.3 noise; GMRES: restart 10, tol 1e-11",
                     "timing": "host wall clock around evolve + synchronize"}
    return out


def bench_sq(reps: int = 20) -> dict:
    """Device S(q) (radial average of |FFT|^2) of a 2D N=1024 field against the
    reference's definition in numpy on the host (utils/sq_from_traj.py)."""
    from chgb import config
    from chgb.sim import CahnHilliard
    oracle = _oracle()
    N = 1024
    p = config.params(2, N, "euler", "landau", dt=0.01, k=1.0, epsilon=0.9)
    sim = CahnHilliard(p, config.init_density(2, N, [0.0], initial_A=1e-2, seed=5))
    sim.evolve(200)
    sim.structure_factor()
    sim.synchronize()
    t0 = time.perf_counter()
    for _ in range(reps):
        sim.structure_factor()
    t_gpu = (time.perf_counter() - t0) / reps
    field = sim.sync().reshape(N, N)
    sim.close()
    t0 = time.perf_counter()
    for _ in range(2):
        oracle.radial_average_sq(field, p.dx)
    t_cpu = (time.perf_counter() - t0) / 2
    return {"value": 1e3 * t_gpu, "unit": "ms per S(q)", "higher_is_better": False,
            "cpu_baseline": {"value": 1e3 * t_cpu, "unit": "ms per S(q)", "cores": 1, "kind": "port",
                             "sample": "numpy FFT + shell average of the same field"},
            "config": {"workload": "S(q) of a 2D N=1024 field (host result: the radially averaged bins)",
                       "timing": "host wall clock, result copied to the host each call"}}


def bench_cufft(N: int = 1024, reps: int = 200) -> dict:
    """A side-by-side timing only, on no product path: cuFFT's FP64 transforms
    (through torch.fft, which calls cuFFT) against the engine's own FFT on the
    2D Landau pseudospectral configuration.  Three figures, all with CUDA
    events on the launching stream, after warm-up:
      * cufft_pair_ms: one D2Z + one Z2D of the N x N field, the two transforms
        a step needs (the reference's CUDA step runs these two,
        src/CUDA/integrators/PseudospectralCUDA.cu:211-222,249-258);
      * cufft_step_ms: a whole FP64 step built on them -- Z2D, f' = -eps psi +
        psi^3, D2Z, psi_hat' = alpha psi_hat - beta f'_hat -- replayed from a
        CUDA graph of 10 steps;
      * chgb_step_ms: this engine's step (row and column passes) on the same field.
    """
    import torch
    from chgb import config
    from chgb.sim import CahnHilliard
    dt, M, k, eps = 0.05, 1.0, 1.0, 0.9
    p = config.params(2, N, "pseudospectral", "landau", dt=dt, k=k, M=M, epsilon=eps)
    rho0 = config.init_density(2, N, [0.0], initial_A=1e-2, seed=SEED)
    stream = torch.cuda.Stream()

    def timed(fn, n):
        a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        torch.cuda.synchronize()
        with torch.cuda.stream(stream):
            a.record(stream)
            fn(n)
            b.record(stream)
        torch.cuda.synchronize()
        return a.elapsed_time(b) / n

    sim = CahnHilliard(p, rho0)
    sim.set_stream(stream.cuda_stream)
    sim.evolve(20)
    sim.synchronize()
    ours = timed(lambda n: sim.evolve(n), reps)
    sim.close()

    with torch.cuda.stream(stream):
        psi = torch.from_numpy(rho0.reshape(N, N)).to("cuda")
        ky = torch.fft.fftfreq(N, d=1.0 / N, dtype=torch.float64, device="cuda") * (2 * np.pi / N)
        kx = torch.arange(N // 2 + 1, dtype=torch.float64, device="cuda") * (2 * np.pi / N)
        q2 = ky[:, None] ** 2 + kx[None, :] ** 2
        den = 1.0 + dt * M * 2.0 * k * q2 * q2
        alpha = (1.0 / den).to(torch.complex128)
        beta = (dt * M * q2 / den).to(torch.complex128)
        psi_hat = torch.fft.rfft2(psi)

    def pair(n):
        for _ in range(n):
            torch.fft.irfft2(torch.fft.rfft2(psi), s=(N, N))

    def step():
        x = torch.fft.irfft2(psi_hat, s=(N, N))
        f = x * x * x - eps * x
        psi_hat.copy_(alpha * psi_hat - beta * torch.fft.rfft2(f))

    pair(5)
    t_pair = timed(pair, reps)
    for _ in range(3):
        with torch.cuda.stream(stream):
            step()
    graph_steps, mode = 10, "CUDA graph of 10 steps"
    try:
        g = torch.cuda.CUDAGraph()
        torch.cuda.synchronize()
        with torch.cuda.graph(g, stream=stream):
            for _ in range(graph_steps):
                step()
        t_step = timed(lambda n: [g.replay() for _ in range(n // graph_steps)], reps)
    except Exception:
        mode = "eager (graph capture unavailable)"
        t_step = timed(lambda n: [step() for _ in range(n)], reps)
    cells = N * N
    return {"value": cells / (ours * 1e-3), "unit": "cell-steps/s", "chgb_step_ms": ours,
            "cufft_pair_ms": t_pair, "cufft_step_ms": t_step, "cufft_step_value": cells / (t_step * 1e-3),
            "chgb_step_vs_cufft_pair": t_pair / ours, "chgb_step_vs_cufft_step": t_step / ours,
            "config": {"workload": f"2D Landau pseudospectral N={N}, dt={dt}, k={k}, M={M}, eps={eps}, FP64; "
                                   "cuFFT side by side (timing only, not a product path)",
                       "cufft_step": mode, "timing": "CUDA events on the launching stream"}}


def bench_driver() -> dict:
    """The drop-in program on the reference's CPU-runnable configuration: 2D
    Landau euler N=64, 10,000 steps, energy every 1000 steps, against the
    oracle stepping the same field on one host thread (no output)."""
    import subprocess
    import tempfile
    from chgb import config
    oracle = _oracle()
    toml = ("steps = 10000\nprint_every = 1000\nprint_trajectory_every = 0\nprint_last_every = 10000\n"
            "N = 64\ndt = 0.01\ndx = 1.0\nk = 1.0\ninitial_density = 0.0\nfree_energy = \"landau\"\n"
            "seed = 12345\nintegrator = \"euler\"\n[landau]\nepsilon = 0.9\n")
    exe = REPO / "cahn-hilliard_gb300" / "lib" / "ch_2D"

    def run(text: str) -> float:
        with tempfile.TemporaryDirectory() as d:
            (Path(d) / "input.toml").write_text(text)
            t0 = time.perf_counter()
            subprocess.run([str(exe), "input.toml"], cwd=d, check=True, capture_output=True, timeout=300)
            return time.perf_counter() - t0

    run(toml)   # warm the file cache
    t_gpu = run(toml)
    # the same run with no steps: process start, CUDA context, init and output
    t_zero = run(toml.replace("steps = 10000", "steps = 0").replace("print_last_every = 10000",
                                                                     "print_last_every = 0"))
    p = config.params(2, 64, "euler", "landau", dt=0.01, k=1.0, epsilon=0.9)
    ref = oracle.OracleSim(p, config.init_density(2, 64, [0.0], initial_A=1e-2, seed=12345))
    t0 = time.perf_counter()
    ref.step(10000)
    t_cpu = time.perf_counter() - t0
    ref.close()
    return {"value": t_gpu, "unit": "s per run", "higher_is_better": False, "zero_step_run_s": t_zero,
            "steps_s": t_gpu - t_zero,
            "cpu_baseline": {"value": t_cpu, "unit": "s per run (steps only)", "cores": 1, "kind": "port",
                             "sample": "the oracle's 10,000 steps of the same field, no output"},
            "config": {"workload": "ch_2D on 2D Landau euler N=64, dt=0.01, 10,000 steps, energy every 1000 steps, "
                                   "last configuration at the end",
                       "timing": "wall clock of the whole process: start, CUDA context, init, steps, output files"}}


def main() -> None:
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=10)
    ap.add_argument("--warmup", type=int, default=3)
    ap.add_argument("--impl", default="chgb", choices=["chgb", "reference"])
    ap.add_argument("--workload", default=HEADLINE, choices=sorted(WORKLOADS))
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline leg")
    ap.add_argument("--only-headline", action="store_true")
    ap.add_argument("--kernel-variant", type=int, default=0, choices=[0, 1, 2, 3, 4, 5],
                    help="euler kernel variant: 0 timed at create (default), 1 fused, 2 split, "
                         "3 two steps per launch (small 2D boxes), 4 the box resident in one cluster (2D N=32, 64), "
                         "5 split in block fixed point (2D/3D Landau)")
    ap.add_argument("--aux", choices=["batch", "adjoint_euler", "adjoint_pseudospectral", "psmob", "sq", "driver",
                                      "cufft"],
                    help="run one auxiliary workload alone and print its JSON (for profiling)")
    ap.add_argument("--aux-steps", type=int, default=0, help="time steps of the --aux workload (0: its default)")
    args = ap.parse_args()
    global KERNEL_VARIANT
    KERNEL_VARIANT = args.kernel_variant
    if args.aux:
        if args.aux == "batch":
            out = bench_batch(args.aux_steps or 200)
        elif args.aux == "psmob":
            out = bench_psmob(args.aux_steps or 200)
        elif args.aux == "sq":
            out = bench_sq()
        elif args.aux == "driver":
            out = bench_driver()
        elif args.aux == "cufft":
            out = bench_cufft()
        else:
            integ = args.aux.split("_", 1)[1]
            out = bench_adjoint(integ, steps=args.aux_steps) if args.aux_steps else bench_adjoint(integ)
        print(json.dumps(out))
        return

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    w = WORKLOADS[args.workload]
    base = {"metric": "cell-steps/s (FP64)", "unit": "cell-steps/s", "n_gpus": world, "steps": args.steps,
            "warmup": args.warmup, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f64", "data": "synthetic (seeded drand48 field, the reference's initialisation)"}

    if args.impl == "reference":
        if rank != 0:
            return
        cpu = bench_cpu(args.workload)
        line = dict(base)
        line.update({"impl": "reference", "value": cpu["value"], "ms_per_step": None,
                     "config": workload_config(args.workload),
                     "cpu_baseline": cpu,
                     "e2e": {"value": cpu["value"], "unit": "cell-steps/s", "h2d_bytes_per_step": 0,
                             "d2h_bytes_per_step": 0}})
        print(json.dumps(line))
        return

    import torch
    if world > 1:
        import torch.distributed as dist
        local = int(os.environ.get("LOCAL_RANK", "0"))
        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
    # replicas only: every rank runs its own box, no collective on the data path
    res = bench_gpu(args.workload, args.steps, args.warmup, with_e2e=True)
    value = res["value"]
    if world > 1:
        ms = max_over_ranks(res["ms_per_step"], "cuda")
        value = whole_job_rate(w["N"] ** w["dims"] * INTERVAL, world, ms / 1e3)
        res["ms_per_step"] = ms
    if rank != 0:
        return
    line = dict(base)
    line.update({"value": value, "ms_per_step": res["ms_per_step"], "config": res["config"],
                 "roofline": res["roofline"], "e2e": res["e2e"], "gpu_launches": res["gpu_launches"],
                 "clocks": res["clocks"]})
    for key in ("fp64_roofline", "alu_roofline"):
        if key in res:
            line[key] = res[key]
    if not args.only_headline:
        subs = {}
        for other in WORKLOADS:
            if other == args.workload:
                continue
            try:
                r = bench_gpu(other, max(3, args.steps // 2), args.warmup, with_e2e=False, ranks=False)
                subs[other] = {"value": r["value"], "roofline": r["roofline"], "config": r["config"],
                               **{k: r[k] for k in ("fp64_roofline", "alu_roofline") if k in r}}
            except Exception as e:  # a workload whose integrator is unavailable is reported, not fatal
                subs[other] = {"error": str(e)}
        try:
            subs["batch2d_256"] = bench_batch(200)
        except Exception as e:
            subs["batch2d_256"] = {"error": str(e)}
        for integ in ("euler", "pseudospectral"):
            try:
                subs[f"adjoint2d_N256_{integ}"] = bench_adjoint(integ)
            except Exception as e:
                subs[f"adjoint2d_N256_{integ}"] = {"error": str(e)}
        for key, fn in (("pseudospectral_mobility", bench_psmob), ("structure_factor_2d_N1024", bench_sq),
                        ("driver_config_N64", bench_driver), ("cufft_side_by_side_2d_N1024", bench_cufft)):
            try:
                subs[key] = fn()
            except Exception as e:
                subs[key] = {"error": str(e)}
        line["workloads"] = subs
    if not args.no_cpu:
        line["cpu_baseline"] = bench_cpu(args.workload)
    print(json.dumps(line))


if __name__ == "__main__":
    main()
