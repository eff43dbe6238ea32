#!/usr/bin/env python3
"""Benchmark of the GB300 tetra-mesh step: prints ONE JSON line.

Workload (default): the large plain cell — Kuhn sphere of radius 64 (6,594,816 tetra,
1,138,197 nodes), Mooney-Rivlin C10 = 5e-4, C01 = 1e-4, K = 1e-2 with the finite-strain
viscoplastic law (yield 2e-4, viscosity 5e-2), rigid substrate, spherical indenter of radius 16
descending 1e-4 per step, damping 1e-2, FP32 kernels. A "step" is one time step of the cell.

  value      tetra-steps/s over --steps steps with the state resident in HBM, timed by CUDA
             events on the library's stream (nfx_time_steps); whole job over all ranks.
  e2e        the same metric through the C ABI with host buffers: per output interval of 100
             steps the indenter positions are uploaded from pinned host memory (the reference's
             per-step beforeTimeStep callable), and the node positions plus the recorded force
             rows come back into pinned host memory (the reference's writeVTK readback) through
             output snapshots (nfx_snapshot) whose copies run while the next interval computes;
             the host waits for every interval's output.
  roofline   the element pass (dominant kernel): algorithmic bytes per launch / its average
             launch duration, from --tet-launches back-to-back launches between two CUDA events
             (nfx_profile_tet_pass), against MEASURED_PEAKS.json hbm_gbs. The per-step
             launch-by-launch event profile (nfx_profile_steps) is reported beside it in config;
             its brackets add the event overhead to every kernel.
  e2e_api    the same metric through the reference-facing Python surface (Simulation with the
             Substrate, Sphere, FiniteStrainViscoplastic and VelocityVerlet plugins): the sphere's
             position is a plain Python callable evaluated on the host for every step and uploaded
             as a position table, and every output interval reads the positions back as
             Simulation.run does (file writing off).
  roofline_1m  the element pass's roofline on the 1M-tetra cell (R = 34, 989,808 tetra).
  batched    the batched population (256 cells, R ~ logU[6, 40], per-cell materials) advanced as
             one batch against looping the plain path over the same cells: sims/s, speed-up,
             tile size per size bucket.
  cpu_baseline  the oracle port of the reference kernels (FP64, OpenMP, all host cores) on a
             bounded sample of the same workload.

--impl reference times the CPU implementation of the path (the oracle port of the reference's
kernels; the reference itself needs an OpenCL runtime that is not installed) on the same
workload and metric. Multi-GPU (torchrun): the single-cell path does not shard, so every rank
runs an independent replica ("replicas only"); value sums the ranks' work over the slowest rank.
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

from nofluidx3d_gb300 import workloads  # noqa: E402

# Algorithmic bytes per tetra-step of the element pass, counted as the unique state a fused
# schedule must stream from HBM per step: connectivity 16 + Dm^-1 36 + V0 4 = 56 B; the
# viscoplastic state adds Fp 36 read + 36 written and the plastic strain 4 + 4 = 80 B.
ELEM_BYTES = {"nh": 56.0, "mr": 56.0, "mr_vp": 136.0}
# Per node and step: position, velocity and previous force, each 12 B read + 12 B written.
NODE_BYTES = 72.0


def load_peaks() -> dict:
    p = os.path.join(ROOT, "MEASURED_PEAKS.json")
    if os.path.exists(p):
        with open(p) as f:
            d = json.load(f)
        return {"hbm_gbs": float(d["hbm_gbs"]), "source": "measured"}
    return {"hbm_gbs": 6800.0, "source": "fallback"}


def profile_figure(workload_key: str, name: str) -> float | None:
    """A per-tetra figure of the element pass (a "name: value" line) from the committed ncu
    summary of the workload, if any."""
    p = os.path.join(ROOT, "profiles", f"tet_pass_{workload_key}.md")
    if not os.path.exists(p):
        return None
    for line in open(p):
        if line.startswith(name + ":"):
            try:
                return float(line.split(":", 1)[1].split()[0])
            except ValueError:
                return None
    return None


def load_traffic(workload_key: str) -> float | None:
    """DRAM bytes per tetra of the element pass from the committed ncu summary, if any."""
    return profile_figure(workload_key, "dram_bytes_per_tetra")


def fp32_rate(flops_per_tet: float | None, nt: int, tet_ms: float, device: int, clk: dict) -> dict | None:
    """Achieved FP32 rate of the element pass: ncu-counted FP32 FLOPs per tetra (2 per FFMA, 1 per
    FADD/FMUL) x tetra / its average launch time, against the nominal FMA peak of the device
    (SMs x 128 FP32 lanes x 2 FLOP x maximum SM clock)."""
    if flops_per_tet is None:
        return None
    import torch

    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = (clk or {}).get("sm_max_mhz") or 2070.0
    peak = sms * 128 * 2 * mhz * 1e6 / 1e12
    achieved = flops_per_tet * nt / (tet_ms / 1e3) / 1e12
    return {"flops_per_tetra": flops_per_tet, "achieved": achieved, "peak": peak, "unit": "TFLOP/s",
            "frac": achieved / peak, "peak_source": "nominal"}


class ClockSampler:
    """nvidia-smi clocks and throttle reasons, sampled every 200 ms during the timed region."""

    FIELDS = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
              "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
              "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, gpu_index: int):
        self.gpu = gpu_index
        self.proc = None
        self.lines: list[str] = []
        self.thread = None

    def start(self):
        try:
            self.proc = subprocess.Popen(
                ["nvidia-smi", f"--id={self.gpu}", f"--query-gpu={self.FIELDS}", "--format=csv,noheader,nounits",
                 "-lms", "200"], stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
        except (OSError, FileNotFoundError):
            self.proc = None
            return
        self.thread = threading.Thread(target=self._read, daemon=True)
        self.thread.start()

    def _read(self):
        for line in self.proc.stdout:
            self.lines.append(line.strip())

    def stop(self) -> dict | None:
        if self.proc is None:
            return None
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except subprocess.TimeoutExpired:
            self.proc.kill()
        if self.thread:
            self.thread.join(timeout=2)
        sm, smax, reasons = [], 0.0, set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for ln in self.lines:
            parts = [p.strip() for p in ln.split(",")]
            if len(parts) < 9:
                continue
            try:
                sm.append(float(parts[1]))
                smax = max(smax, float(parts[2]))
            except ValueError:
                continue
            for n, v in zip(names, parts[5:9]):
                if v.lower().startswith("active"):
                    reasons.add(n)
        if not sm:
            return None
        return {"sm_mhz": statistics.median(sm), "sm_max_mhz": smax, "reasons": sorted(reasons), "samples": len(sm)}


def dist_setup():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    if world > 1:
        import torch
        import torch.distributed as dist

        torch.cuda.set_device(local)
        dist.init_process_group("nccl")
        return world, rank, local, dist
    return 1, 0, 0, None


def reduce_max(dist, x: float, local: int) -> float:
    if dist is None:
        return x
    import torch

    t = torch.tensor([x], dtype=torch.float64, device=f"cuda:{local}")
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def barrier(dist, local: int):
    if dist is not None:
        import torch

        dist.barrier(device_ids=[local])
        torch.cuda.synchronize(local)


def cpu_baseline(w, sample_seconds: float, threads: int = 0) -> dict:
    """The oracle port (FP64, OpenMP over work-items) on a bounded number of whole time steps."""
    import oracle as O
    from tests.helpers import oracle_problem

    mesh = w.mesh()
    st = O.State(oracle_problem(w, mesh), "f64")
    th = threads or O.max_threads()
    t0 = time.perf_counter()
    st.run(1, parallel=True, threads=th)  # warm-up (page-in, thread pool)
    one = time.perf_counter() - t0
    n = max(1, int(sample_seconds / max(one, 1e-6)))
    t0 = time.perf_counter()
    st.run(n, parallel=True, threads=th)
    dt = time.perf_counter() - t0
    return {"value": mesh.num_tetra * n / dt, "unit": "tetra-steps/s", "cores": th, "kind": "port",
            "sample": f"{n} whole time steps of the {w.name} cell ({mesh.num_tetra} tetra), FP64, "
                      f"{th} OpenMP threads, after 1 warm-up step"}


def run_reference(args):
    world, rank, local, dist = dist_setup()
    if rank != 0:
        return
    w = workloads.WORKLOADS[args.workload]()
    import oracle as O
    from tests.helpers import oracle_problem

    mesh = w.mesh()
    st = O.State(oracle_problem(w, mesh), "f64")
    th = O.max_threads()
    t0 = time.perf_counter()
    for _ in range(args.warmup):  # the requested warm-up, unless it would take more than a third of the budget
        st.run(1, parallel=True, threads=th)
        if time.perf_counter() - t0 > args.reference_seconds / 3:
            break
    budget = args.reference_seconds
    done, t0 = 0, time.perf_counter()
    while done < args.steps and (time.perf_counter() - t0) < budget:
        st.run(1, parallel=True, threads=th)
        done += 1
    dt = time.perf_counter() - t0
    val = mesh.num_tetra * done / dt
    line = {
        "impl": "reference", "metric": METRIC, "value": val, "unit": "tetra-steps/s", "n_gpus": world,
        "steps": done, "warmup": args.warmup, "ms_per_step": 1e3 * dt / max(done, 1),
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
        "config": bench_config(w, mesh.num_tetra, mesh.num_points, world),
        "implementation": "oracle port of the reference's OpenCL kernels, OpenMP",
        "cpu_baseline": {"value": val, "unit": "tetra-steps/s", "cores": th, "kind": "port",
                         "sample": f"{done} whole time steps (of {args.steps} requested, capped at {budget:.0f} s)"},
        "e2e": {"value": val, "unit": "tetra-steps/s", "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


METRIC = "tetra-steps/s + % HBM peak, 1 GB300"


def bench_config(w, nt: int, npn: int, world: int) -> dict:
    """The workload description both arms print (identical for the same workload)."""
    mb = (ELEM_BYTES[w.material] * nt + NODE_BYTES * npn) / 1e6
    l2 = (f"inputs larger than L2: {mb:.0f} MB of algorithmic state streamed per step vs 129 MB L2" if mb > 129 else
          f"L2-resident: {mb:.0f} MB of algorithmic state per step fits the 129 MB L2 (no flush; a small-cell "
          "latency figure, not a bandwidth one)")
    return {"workload": w.name, "tets": nt, "nodes": npn, "parallelism": "replicas" if world > 1 else "single", "l2": l2}


def batched_measure(args, world, rank, local, dist, steps: int, warmup: int) -> dict | None:
    """Batched population (256 cells, radius log-uniform in [6, 40] unless --batch-rmin/--batch-rmax
    say otherwise, per-cell materials): steps/s of one batch advancing every cell, against looping
    the plain path over the same cells (each cell's plain step time measured on that cell through
    nfx_step in CUDA-graph chunks, summed). sims/s = cells / (20k steps' time). Under torchrun the
    cells are split across ranks by LPT on their tetra counts (no data-path collective); times are
    the maximum over ranks. Returns the JSON line on rank 0 (None elsewhere)."""
    from nofluidx3d_gb300.core import Batch, CellSim
    from nofluidx3d_gb300.mesh import mesh_counts
    from nofluidx3d_gb300.shard import lpt_partition

    r_range = (args.batch_rmin, args.batch_rmax)
    all_cells = workloads.batched_cells(args.batch_cells, seed=0, r_range=r_range)
    n_all = len(all_cells)
    nt_all = sum(mesh_counts(w.radius)[1] for w in all_cells)
    mine = lpt_partition([mesh_counts(w.radius)[1] for w in all_cells], world)[rank]
    cells = [all_cells[i] for i in mine]
    t0 = time.perf_counter()
    meshes = [w.mesh() for w in cells]
    t_mesh = time.perf_counter() - t0
    t0 = time.perf_counter()
    b = Batch(local, tile_tets=args.batch_tile)
    for w, m in zip(cells, meshes):
        w.add_to_batch(b, m)
    b.set_record(1, 100, warmup + steps + 60)
    b.finalize()
    t_setup = time.perf_counter() - t0
    b.time_steps(max(warmup, 50))  # at least one 50-step chunk, so its graph exists before timing
    barrier(dist, local)
    ms = reduce_max(dist, b.time_steps(steps), local)
    batch_step_ms = ms / steps
    status = b.status()
    cell_status = b.cell_status()
    info = b.info()
    b.close()
    # looped plain path: each cell alone, a short timed run per cell. The cells' handles are set up
    # on host threads (each builds its own plan in native code), then timed one after another.
    from concurrent.futures import ThreadPoolExecutor

    def make(wm):
        s = CellSim(local)
        wm[0].configure(s, wm[1], max_rows=4)
        return s

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        sims = list(ex.map(make, zip(cells, meshes)))
    plain_ms = []
    for s in sims:
        s.time_steps(100)  # warm-up that also captures the cell's 100-step graph
        plain_ms.append(s.time_steps(args.loop_steps) / args.loop_steps)
        s.close()
    loop_step_ms = reduce_max(dist, sum(plain_ms), local)
    status = int(reduce_max(dist, float(status), local))
    n_bad = int(reduce_max(dist, float((cell_status != 0).sum()), local))
    if rank != 0:
        return None
    n, nt = n_all, nt_all
    sim_steps = 20000
    line = {
        "metric": f"batched sims/s ({n} cells, 20k steps)", "value": n / (batch_step_ms * sim_steps / 1e3),
        "unit": "sims/s", "n_gpus": world, "steps": steps, "warmup": warmup, "ms_per_step": batch_step_ms,
        "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": {"workload": f"batched {n} cells R~logU[{r_range[0]:g},{r_range[1]:g}], per-cell VP materials",
                   "tets": nt,
                   "tile_tets": info["tile_tets"], "buckets": info["buckets"],
                   "autotune_ms_per_10_steps": info["tuning"],
                   "batch_tetra_steps_per_s": nt / (batch_step_ms / 1e3),
                   "looped_plain_ms_per_step": loop_step_ms,
                   "looped_plain_sims_per_s": n / (loop_step_ms * sim_steps / 1e3),
                   "speedup_vs_looped_plain": loop_step_ms / batch_step_ms,
                   "looped_plain_steps_per_cell": args.loop_steps,
                   "mesh_gen_s": t_mesh, "setup_s": t_setup, "status": status,
                   "cells_with_status_max_rank": n_bad, "parallelism": f"cells sharded by LPT over {world} GPU(s)"},
    }
    return line


def run_batched(args):
    world, rank, local, dist = dist_setup()
    line = batched_measure(args, world, rank, local, dist, args.steps, args.warmup)
    if line is not None:
        print(json.dumps(line), flush=True)


def e2e_api(w, mesh, local: int, steps: int) -> dict:
    """The workload through the reference-facing Python surface: Simulation (built on the same
    mesh), Substrate, a Sphere whose position is a plain Python callable (evaluated on the host
    for every step, uploaded as a per-step table), FiniteStrainViscoplastic and VelocityVerlet,
    and Simulation.run's output loop with file writing off: every interval reads the positions
    back and evaluates the recorded quantities (time, indentation, indenter force). Wall clock
    over run(), after one untimed interval that captures the step graph."""
    import tempfile

    from nofluidx3d_gb300.interactions import FiniteStrainViscoplastic, Sphere
    from nofluidx3d_gb300.Simulation import Simulation
    from nofluidx3d_gb300.TetraCell import TetraCell

    interval = w.record_every
    frames = max(1, steps // interval)
    sph = w.contacts(mesh)[w.record_contact]
    p0, v = sph["p0"], sph["v"]
    R = w.radius
    with tempfile.TemporaryDirectory() as td:
        cfg = {"gpu": local, "RhoSI": 1.0, "SimulationTimeSI": float(frames * interval), "VTKFramesTotal": frames,
               "OutputDir": td + "/", "InitialDistance": w.initial_distance(mesh), "MoveTimeSI": 1e30,
               "VelocitySI": w.speed, "SphereRadiusSI": w.sphere_radius,
               "CELL": {"RadiusSI": R, "RadiusSIM": R, "YoungsModulusSI": 1e-2, "PoissonRatio": 0.3}}
        sim = Simulation(cfg, verbose=False, cell=TetraCell.from_arrays(mesh.points, mesh.tets, radius=R))
        sim.setInteractionSubstrate()
        sphere = Sphere(sph["radius"], lambda t: p0 - v * t, sph["k"])
        sim.register(sphere)
        sim.register(FiniteStrainViscoplastic(*w.vp_params()))
        sim.setInteractionVelocityVerlet(damping=w.xi)
        sim.recordedQuantities.append(lambda: v * sim.time)
        sim.recordedQuantities.append(lambda: sim.handle.indenter_force(sphere.contactId))
        sim._advance(interval)
        sim.handle.sync()
        t0 = time.perf_counter()
        data = sim.run(writeStress=False, writePressure=False, write=False)
        dt = time.perf_counter() - t0
        status = sim.handle.status()
        sim.close()
    n = frames * interval
    return {"value": mesh.num_tetra * n / dt, "unit": "tetra-steps/s", "steps": n, "interval": interval,
            "outputs": frames + 1, "h2d_bytes_per_step": 8.0 * (interval + 1) / interval,
            "d2h_bytes_per_step": (frames + 1) * (8.0 * 3 * mesh.num_points + 8.0) / n,
            "path": "Simulation.run(write=False): Python sphereFunc -> position tables, positions read back "
                    "every interval, force via the handle's readout",
            "final_force": float(data[-1, 2]), "status": status}


def roofline_1m(local: int, launches: int, peak: float) -> dict:
    """The element pass on the 1M-tetra cell (R = 34 plain-large construction): algorithmic bytes
    per launch over its average duration across back-to-back launches, after 300 steps."""
    from nofluidx3d_gb300.core import CellSim

    w = workloads.plain_large_1m()
    mesh = w.mesh()
    sim = CellSim(local)
    w.configure(sim, mesh, max_rows=40)
    sim.time_steps(300)
    step_ms = sim.time_steps(2000) / 2000
    ms = sim.profile_tet_pass(launches)
    sim.close()
    nt = mesh.num_tetra
    achieved = ELEM_BYTES[w.material] * nt / (ms / 1e3) / 1e9
    return {"workload": w.name, "tets": nt, "tet_pass_ms": ms, "launches_timed": launches, "achieved": achieved,
            "peak": peak, "unit": "GB/s", "frac": achieved / peak, "ms_per_step": step_ms,
            "tetra_steps_per_s": nt / (step_ms / 1e3),
            "step_frac": (ELEM_BYTES[w.material] * nt + NODE_BYTES * mesh.num_points) / (step_ms / 1e3) / 1e9 / peak}


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=8000,
                    help="timed steps (8000 at R=64: about 2 s, ten clock samples)")
    ap.add_argument("--warmup", type=int, default=200)
    ap.add_argument("--impl", default="nfx", choices=["nfx", "reference"])
    ap.add_argument("--workload", default="plain-large", choices=sorted(workloads.WORKLOADS))
    ap.add_argument("--profile-steps", type=int, default=20)
    ap.add_argument("--tet-launches", type=int, default=20,
                    help="back-to-back element-pass launches timed for the roofline")
    ap.add_argument("--e2e-steps", type=int, default=1000)
    ap.add_argument("--cpu-seconds", type=float, default=15.0)
    ap.add_argument("--reference-seconds", type=float, default=90.0)
    ap.add_argument("--no-cpu-baseline", action="store_true")
    ap.add_argument("--batched", action="store_true", help="batched population instead of one cell")
    ap.add_argument("--batch-cells", type=int, default=256)
    ap.add_argument("--batch-tile", type=int, default=0, help="0: autotune")
    ap.add_argument("--loop-steps", type=int, default=200,
                    help="steps per cell when timing the looped plain path (multiples of 100 run as CUDA graphs)")
    ap.add_argument("--batch-rmin", type=float, default=6.0)
    ap.add_argument("--batch-rmax", type=float, default=40.0)
    ap.add_argument("--batch-steps", type=int, default=200, help="timed batch steps in the default run")
    ap.add_argument("--no-batched", action="store_true", help="skip the batched measurement of the default run")
    ap.add_argument("--no-api", action="store_true", help="skip the Simulation-surface e2e_api measurement")
    ap.add_argument("--no-1m", action="store_true", help="skip the 1M-tetra roofline")
    ap.add_argument("--clock-window-s", type=float, default=2.0,
                    help="untimed steps run just before the timed region while clocks are sampled")
    args = ap.parse_args()
    if args.warmup < 3:
        ap.error("--warmup must be >= 3")
    if args.impl == "reference":
        return run_reference(args)
    if args.batched:
        return run_batched(args)

    world, rank, local, dist = dist_setup()
    from nofluidx3d_gb300.core import CellSim

    w = workloads.WORKLOADS[args.workload]()
    mesh = w.mesh()
    # force rows for every step this process runs (the clock window's length depends on the step
    # time: up to about 2 M steps for the smallest cell)
    total = args.warmup + args.steps + args.profile_steps + args.e2e_steps + 400 + 2_000_000
    sim = CellSim(local)
    w.configure(sim, mesh, max_rows=total // w.record_every + 2)
    nt, npn = mesh.num_tetra, mesh.num_points

    # warm-up; the library captures its 100-step CUDA graph on the first call of >= 100 steps, so
    # a short warm-up is followed by one untimed 100-step chunk that captures it
    sim.time_steps(args.warmup)
    if args.warmup < 100:
        sim.time_steps(100)
    # The clock sampler (nvidia-smi, 200 ms period) runs from the start of an untimed window of at
    # least --clock-window-s seconds of the same steps through the end of the timed region, so
    # that a short timed region still has clock samples under load around it.
    clocks = ClockSampler(local)
    clocks.start()
    # the window stays within the workload's own duration (w.steps), so that the cell is still in
    # its physical range when the timed steps and the e2e intervals that follow run
    window_ms = 0.0
    after = args.steps + args.profile_steps + args.e2e_steps + 400
    while window_ms < 1e3 * args.clock_window_s and sim.time + 1000 + after <= w.steps:
        window_ms += sim.time_steps(1000)
    barrier(dist, local)
    ms = sim.time_steps(args.steps)
    barrier(dist, local)
    clk = clocks.stop()
    if clk is not None:
        clk["window"] = f"{window_ms / 1e3:.1f} s of the same steps just before the timed region, and the timed region"
    ms = reduce_max(dist, ms, local)
    value = world * nt * args.steps / (ms / 1e3)

    # per-kernel CUDA-event profile of the element and node passes, then the element pass alone
    # over back-to-back launches (its effects undone)
    tet_ms, node_ms = sim.profile_steps(args.profile_steps)
    tet_avg = tet_ms / args.profile_steps
    tet_launch_ms = sim.profile_tet_pass(args.tet_launches)
    elem_bytes = ELEM_BYTES[w.material] * nt
    achieved = elem_bytes / (tet_launch_ms / 1e3) / 1e9
    peaks = load_peaks()
    traffic_per_tet = load_traffic(args.workload)
    flops_per_tet = profile_figure(args.workload, "fp32_flops_per_tetra")

    # end to end through the C ABI with pinned host buffers
    import torch

    # two sets of pinned host buffers: the host reads interval k's output (snapshot) while the
    # device runs interval k + 1
    pos_host = [torch.empty(3 * npn, dtype=torch.float64, pin_memory=True).numpy() for _ in range(2)]
    rows_host = [torch.empty((total // w.record_every + 2, 3), dtype=torch.float64, pin_memory=True).numpy()
                 for _ in range(2)]
    tab_host = [torch.empty(w.record_every, dtype=torch.float64, pin_memory=True).numpy() for _ in range(2)]
    c = w.contacts(mesh)[w.record_contact]
    intervals = max(1, args.e2e_steps // w.record_every)
    # the first snapshot creates the copy stream, its events and the staging buffer: not timed
    sim.snapshot(pos_host[1], rows_host[1])
    sim.snapshot_wait()
    barrier(dist, local)
    sim.sync()
    t0 = time.perf_counter()
    n_rows = 0
    d2h_bytes = 0.0
    for k in range(intervals):
        t = sim.time
        tt = np.arange(t, t + w.record_every, dtype=np.float64)
        tab_host[k % 2][:] = c["p0"] - c["v"] * tt  # the host-side position callable
        sim.set_contact_table(w.record_contact, t, tab_host[k % 2])
        sim.step(w.record_every)
        if k > 0:
            sim.snapshot_wait()  # interval k - 1's positions and force rows are on the host
            _ = rows_host[(k - 1) % 2][n_rows - 1] if n_rows else None
        n_rows = sim.snapshot(pos_host[k % 2], rows_host[k % 2])
        d2h_bytes += 8.0 * 3 * npn + 24.0 * min(n_rows, rows_host[0].shape[0])
    sim.snapshot_wait()
    sim.sync()
    e2e_s = reduce_max(dist, time.perf_counter() - t0, local)
    e2e_steps = intervals * w.record_every
    e2e_val = world * nt * e2e_steps / e2e_s
    h2d = 8.0 * w.record_every * intervals / e2e_steps + 16.0 / w.record_every
    d2h = d2h_bytes / e2e_steps
    status = sim.status()
    sim.close()

    api = None if args.no_api else e2e_api(w, mesh, local, args.e2e_steps)
    r1m = None if args.no_1m else roofline_1m(local, args.tet_launches, peaks["hbm_gbs"])
    batched = None
    if not args.no_batched:
        batched = batched_measure(args, world, rank, local, dist, args.batch_steps, 50)

    if rank != 0:
        barrier(dist, local)
        return
    cpu = None
    if not args.no_cpu_baseline:
        try:
            cpu = cpu_baseline(w, args.cpu_seconds)
        except Exception as e:  # the baseline is reported, not required
            cpu = {"value": None, "error": str(e)}
    line = {
        "metric": METRIC, "value": value, "unit": "tetra-steps/s", "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms / args.steps, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "f32", "data": "synthetic",
        "config": bench_config(w, nt, npn, world),
        "diagnostics": {
                   "step_bytes_per_tetra": ELEM_BYTES[w.material] + NODE_BYTES * npn / nt,
                   "step_gbs": (ELEM_BYTES[w.material] * nt + NODE_BYTES * npn) / (ms / args.steps / 1e3) / 1e9,
                   "tet_pass_ms": tet_launch_ms, "tet_pass_ms_bracketed": tet_avg,
                   "node_pass_ms_bracketed": node_ms / args.profile_steps, "status": status},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peaks["hbm_gbs"], "unit": "GB/s",
                     "frac": achieved / peaks["hbm_gbs"], "peak_source": peaks["source"],
                     "kernel": "k_tet_pass (element pass)", "launches_timed": args.tet_launches,
                     "algorithmic_bytes_per_launch": elem_bytes,
                     "traffic": None if traffic_per_tet is None else traffic_per_tet * nt},
        "fp32": fp32_rate(flops_per_tet, nt, tet_launch_ms, local, clk),
        "cpu_baseline": cpu,
        "e2e": {"value": e2e_val, "unit": "tetra-steps/s", "h2d_bytes_per_step": h2d, "d2h_bytes_per_step": d2h},
        "e2e_api": api,
        "roofline_1m": r1m,
        "batched": None if batched is None else {
            "sims_per_s": batched["value"], "ms_per_step": batched["ms_per_step"], "steps": batched["steps"],
            **{k: batched["config"][k] for k in ("workload", "tets", "buckets", "tile_tets", "batch_tetra_steps_per_s",
                                                 "looped_plain_ms_per_step", "looped_plain_sims_per_s",
                                                 "speedup_vs_looped_plain", "autotune_ms_per_10_steps", "status",
                                                 "cells_with_status_max_rank", "setup_s")}},
        "gpu_launches": 2 * args.steps + (args.steps + 99) // 100,
        "clocks": clk,
    }
    print(json.dumps(line), flush=True)
    barrier(dist, local)


if __name__ == "__main__":
    main()
