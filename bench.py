"""Benchmark of the GB300 MONKI transport hot path.

Workload: the layered-cloud scene (polarized I/Q/U with layer-AMF paths): 30 x 20
periodic 1 km columns, 34 layers plus vacuum, Rayleigh 0.70 + O3 0.30 + aerosol 0.20
(g 0.70, SSA 0.92) + a 2-3 km cloud slab of optical depth 10 (g 0.85, SSA 0.9999),
SZA 30, views (VZA, RAA) = (0,0), (30,90), (60,180), albedo 0.05, FP32 transport with
FP64 per-round tallies, 20,000 photons per column per round. One step = one statistical
round (12,000,000 photon histories) through the transport kernel and the FP64 flush.

Printed JSON (one line, rank 0):
  value      scatters/s with the scene resident on the device, from CUDA events on the
             session stream around each step (L2 flushed between steps);
  e2e        the same metric through the public API (``CUDA.prepare`` + ``run_batches``),
             wall clock, including the table upload and every round's tally copy-out;
  roofline   the transport kernel's algorithmic bytes per launch (16 B per cell visit on
             the free path and the detector rays, 8 B per FP32 tally read-modify-write)
             over its event-timed duration, against the measured HBM copy bandwidth;
  cpu_baseline  the FP64 CPU restatement of the reference transport (oracle) on a bounded
             sample of the same round, on every host core.

``--impl reference`` times that CPU restatement alone (the reference's Fortran transport
cannot be compiled here), with the same metric and configuration.
"""

from __future__ import annotations

import argparse
import ctypes
import json
import os
import re
import statistics
import subprocess
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "monki-gpu_gb300"))

METRIC = "time to SE/|I|<1% per scene, plain vs importance-guided MC on 1 GB300; scatters/s"
UNIT = "scatters/s"
PHOTONS_PER_COLUMN = 20_000
WORKLOAD = "layered-cloud 30x20x35, I/Q/U + layer AMF, 20000 photons/column/round"
STATE_BYTES = 64  # one event's photon state records read by the peel kernel
CELL_BYTES = 16  # one cell record (beta + cumulative species fractions)
TALLY_BYTES = 32  # one 128-bit tally atomic: 16 B read + 16 B written in L2


def peaks():
    path = ROOT / "MEASURED_PEAKS.json"

    if path.is_file():
        data = json.loads(path.read_text())
        return float(data["hbm_gbs"]), "measured"

    return 6800.0, "fallback"


def recorded_traffic():
    """Per-launch DRAM bytes of the transport kernel from the committed ncu summary."""

    path = ROOT / "profiles" / "transport_kernel_layered_cloud.md"

    if not path.is_file():
        return None

    match = re.search(r"traffic_bytes_per_launch:\s*([0-9.eE+]+)", path.read_text())
    return float(match.group(1)) if match else None


class Clocks:
    """nvidia-smi samples of SM clock and throttle reasons during the timed region."""

    QUERY = (
        "index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
        "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
        "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap"
    )

    def __init__(self, device: int):
        self.device = device
        self.process = None
        self.path = Path(os.environ.get("TMPDIR", "/tmp")) / f"monki_clocks_{os.getpid()}.csv"

    def __enter__(self):
        try:
            self.process = subprocess.Popen(
                ["nvidia-smi", f"--id={self.device}", f"--query-gpu={self.QUERY}", "--format=csv,noheader,nounits", "-lms", "200"],
                stdout=open(self.path, "w"),
                stderr=subprocess.DEVNULL,
            )
        except (FileNotFoundError, OSError):
            self.process = None

        return self

    def __exit__(self, *args):
        if self.process is not None:
            self.process.terminate()
            try:
                self.process.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.process.kill()

    def summary(self):
        if self.process is None or not self.path.is_file():
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"]}

        rows = []

        for line in self.path.read_text().splitlines():
            parts = [p.strip() for p in line.split(",")]

            if len(parts) >= 9:
                rows.append(parts)

        self.path.unlink(missing_ok=True)

        if not rows:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["no samples"]}

        sm = [float(r[1]) for r in rows if r[1].replace(".", "").isdigit()]
        top = [float(r[2]) for r in rows if r[2].replace(".", "").isdigit()]
        names = ("hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap")
        reasons = sorted({name for r in rows for name, flag in zip(names, r[5:9]) if flag.lower() == "active"})
        loaded = sorted(sm)[len(sm) // 2 :] or sm
        return {
            "sm_mhz": statistics.median(loaded) if loaded else None,
            "sm_max_mhz": max(top) if top else None,
            "reasons": reasons,
            "samples": len(rows),
        }


def distributed():
    world = int(os.environ.get("WORLD_SIZE", "1"))
    rank = int(os.environ.get("RANK", "0"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    return world, rank, local


def cpu_baseline(scene, target_seconds: float = 10.0):
    """Scatters/s of the FP64 CPU restatement on a bounded sample of one round."""

    from oracle import oracle

    nmat, nx, ny, nz, angles = scene.shape
    per_round = scene.photons_per_column * nx * ny
    threads = os.cpu_count() or 1
    calibration = max(threads * 64, 4096)
    start = time.perf_counter()
    _, counters = oracle.run(scene.tables, [calibration, 0, 1, 0, 100000, 0, per_round, 1], threads)
    rate = calibration / max(time.perf_counter() - start, 1e-6)
    sample = int(min(per_round - calibration, max(calibration, rate * target_seconds)))
    start = time.perf_counter()
    _, counters = oracle.run(scene.tables, [sample, calibration, 1, 0, 100000, 0, per_round, 1], threads)
    elapsed = time.perf_counter() - start
    return {
        "value": counters["scatters"] / elapsed,
        "unit": UNIT,
        "cores": threads,
        "kind": "port",
        "sample": f"{sample} of the {per_round} photon histories of one round ({elapsed:.1f} s, "
        f"{counters['scatters']} scatters), FP64 C++ restatement of mc.f90 with OpenMP",
    }


def reference_arm(args):
    import monki.scenes as scenes

    world, rank, _ = distributed()

    if rank != 0:
        return 0

    scene = scenes.layered_cloud(PHOTONS_PER_COLUMN, 1)
    from oracle import oracle

    nmat, nx, ny, nz, angles = scene.shape
    per_round = PHOTONS_PER_COLUMN * nx * ny
    threads = os.cpu_count() or 1
    sample = max(threads * 256, 20_000)
    scatters = 0
    elapsed = 0.0

    for step in range(args.warmup + args.steps):
        first = (step * sample) % max(per_round - sample, 1)
        start = time.perf_counter()
        _, counters = oracle.run(scene.tables, [sample, first, 1, 0, 100000, 0, per_round, 1], threads)
        dt = time.perf_counter() - start

        if step >= args.warmup:
            scatters += counters["scatters"]
            elapsed += dt

    value = scatters / elapsed
    line = {
        "impl": "reference",
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": args.gpus,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": elapsed / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f64",
        "data": "synthetic",
        "config": {"workload": WORKLOAD, "step": f"{sample} photon histories of one round on the host cores"},
        "cpu_baseline": {
            "value": value,
            "unit": UNIT,
            "cores": threads,
            "kind": "port",
            "sample": f"{sample} photon histories per step; the reference's Fortran transport needs gfortran, "
            "which is absent, so its FP64 C++ restatement (oracle/) runs instead",
        },
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line))
    return 0


def main():
    parser = argparse.ArgumentParser()
    parser.add_argument("--gpus", type=int, default=1)
    parser.add_argument("--steps", type=int, default=8)
    parser.add_argument("--warmup", type=int, default=3)
    parser.add_argument("--impl", default="gb300", choices=("gb300", "reference"))
    parser.add_argument("--no-cpu-baseline", action="store_true")
    parser.add_argument("--photons-per-column", type=int, default=PHOTONS_PER_COLUMN)
    args = parser.parse_args()

    if args.warmup < 3:
        parser.error("at least 3 warm-up steps are required")

    if args.impl == "reference":
        return reference_arm(args)

    import torch

    import monki.scenes as scenes
    from monki.execution import CUDA, BatchControls
    from monki.execution import native as binding

    world, rank, local = distributed()
    torch.cuda.set_device(local)

    if world > 1:
        import torch.distributed as dist

        dist.init_process_group("nccl")

    def barrier():
        if world > 1:
            torch.distributed.barrier()

        torch.cuda.synchronize()

    ppc = args.photons_per_column
    scene = scenes.layered_cloud(ppc, args.warmup + args.steps)
    nmat, nx, ny, nz, angles = scene.shape
    per_round = ppc * nx * ny
    native = binding.load()
    tables = np.ascontiguousarray(scene.tables)
    err = ctypes.create_string_buffer(4096)
    capacity = max(args.steps, args.warmup)
    handle = native.monki_cuda_create(
        local, tables.ctypes.data_as(binding.F64P), tables.size, capacity, b"precision=fp32", err, len(err)
    )

    if not handle:
        raise RuntimeError(err.value.decode())

    tally_count = int(native.monki_cuda_tally_count(handle))
    out = np.zeros(tally_count * capacity)
    flush = torch.empty(256 * 1024 * 1024 // 4, dtype=torch.float32, device=f"cuda:{local}")
    timing = (ctypes.c_float * 2)()
    counters_before = (ctypes.c_uint64 * 6)()
    counters_after = (ctypes.c_uint64 * 6)()

    def group(first_round, rounds):
        """One round group in one dispatch, as CUDA.run_batches schedules it, with the
        per-stage event timing on. Ranks run disjoint rounds (offset 100000 per rank)."""

        controls = (ctypes.c_uint32 * 8)(
            per_round * rounds, 0, rank * 100000 + first_round, 0, 100000, 1, per_round, rounds
        )

        if native.monki_cuda_run(handle, controls, out.ctypes.data_as(binding.F64P), err, len(err)):
            raise RuntimeError(err.value.decode())

        native.monki_cuda_last_timing(handle, timing)
        return timing[0], timing[1]

    # Warm-up: W rounds, untimed.
    flush.zero_()
    torch.cuda.synchronize()
    group(1, args.warmup)
    native.monki_cuda_counters(handle, counters_before)
    flush.zero_()  # 256 MiB write: the timed group starts with a cold L2
    barrier()

    with Clocks(local) as clocks:
        wall = time.perf_counter()
        kernel_ms, run_ms = group(args.warmup + 1, args.steps)
        barrier()
        wall = time.perf_counter() - wall

    native.monki_cuda_counters(handle, counters_after)
    stage_ms = (ctypes.c_double * 3)()
    stage_launches = (ctypes.c_uint64 * 3)()
    native.monki_cuda_stage_timing(handle, stage_ms, stage_launches)
    delta = [int(a) - int(b) for a, b in zip(counters_after, counters_before, strict=True)]
    scatters, visits_fp, visits_det, updates, photons, launches = delta
    device_seconds = run_ms / 1e3

    if world > 1:
        import torch.distributed as dist

        t = torch.tensor([device_seconds], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(t, op=dist.ReduceOp.MAX)
        device_seconds = float(t.item())
        s = torch.tensor([float(scatters)], device=f"cuda:{local}", dtype=torch.float64)
        dist.all_reduce(s)
        total_scatters = float(s.item())
    else:
        total_scatters = float(scatters)

    native.monki_cuda_close(handle)
    value = total_scatters / device_seconds
    # Roofline of the dominant kernel, the peel stage: per launch, the event state it reads,
    # the cells its detector rays visit and its 128-bit tally atomics, over its event time.
    peel_launches = max(int(stage_launches[1]), 1)
    peel_seconds = stage_ms[1] / 1e3 / peel_launches
    peel_bytes = (STATE_BYTES * scatters + CELL_BYTES * visits_det + TALLY_BYTES * updates) / peel_launches
    peak, peak_kind = peaks()
    achieved = peel_bytes / peel_seconds / 1e9
    stage_total = max(sum(stage_ms), 1e-9)
    stage_share = {name: stage_ms[q] / stage_total for q, name in enumerate(("transit", "peel", "scatter"))}

    # End to end through the public API: prepare (table upload) + every round's copy-out.
    e2e_scene = scenes.layered_cloud(ppc, args.steps)
    torch.cuda.synchronize()
    wall_e2e = time.perf_counter()

    with CUDA(device=local, seed=rank) as backend:
        backend.prepare(e2e_scene)
        batches = backend.run_batches([BatchControls(i, ppc) for i in range(1, args.steps + 1)])
        e2e_scatters = backend.provenance["scatters"]
        e2e_launches = backend.provenance["kernel_launches"]

    wall_e2e = time.perf_counter() - wall_e2e
    assert len(batches) == args.steps
    e2e_value = e2e_scatters * world / wall_e2e
    tally_bytes = tally_count * 8

    if rank != 0:
        if world > 1:
            torch.distributed.destroy_process_group()

        return 0

    line = {
        "metric": METRIC,
        "value": value,
        "unit": UNIT,
        "n_gpus": world,
        "steps": args.steps,
        "warmup": args.warmup,
        "ms_per_step": device_seconds / args.steps * 1e3,
        "higher_is_better": True,
        "scaling": "weak",
        "vs_baseline": None,
        "dtype": "f32",
        "data": "synthetic",
        "config": {
            "workload": WORKLOAD,
            "photons_per_step": per_round,
            "scatters_per_step": scatters / args.steps,
            "l2": "flushed between steps by a 256 MiB device write",
            "parallelism": f"{world} independent round streams" if world > 1 else "1 GPU",
            "wall_s": wall,
        },
        "roofline": {
            "bound": "hbm",
            "kernel": "wf_peel (event peel-off: phase matrix, detector ray, tallies)",
            "achieved": achieved,
            "peak": peak,
            "unit": "GB/s",
            "frac": achieved / peak,
            "traffic": recorded_traffic(),
            "peak_source": peak_kind,
            "algorithmic_bytes_per_launch": peel_bytes,
            "launch_ms": peel_seconds * 1e3,
            "launches": peel_launches,
            "stage_share": stage_share,
        },
        "e2e": {
            "value": e2e_value,
            "unit": UNIT,
            "h2d_bytes_per_step": tables.nbytes / args.steps + 32,
            "d2h_bytes_per_step": tally_bytes,
            "wall_s": wall_e2e,
            "note": "CUDA.prepare (table upload) + run_batches of all steps, tallies copied to host",
        },
        "gpu_launches": launches,
        "e2e_gpu_launches": e2e_launches,
        "clocks": clocks.summary(),
    }

    if not args.no_cpu_baseline:
        line["cpu_baseline"] = cpu_baseline(scenes.layered_cloud(ppc, 1))

    print(json.dumps(line))

    if world > 1:
        torch.distributed.destroy_process_group()

    return 0


if __name__ == "__main__":
    sys.exit(main())
