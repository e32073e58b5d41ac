"""Benchmark of the GB300 on-lattice Monte Carlo hot path.

Workload (the configuration the headline metric is quoted on): the batched
2D Ising ensemble - 512 independent sq/4n replicas with L drawn log-uniform in
[64, 1024] and rounded to a multiple of 32, kT uniform in [1.5, 3.5], int8
spins uniform from the seed, replica exchange between neighbouring
temperatures (of equal-L replicas) every 10 sweeps, 2000 sweeps in all.
One step = 10 sweeps of every replica plus one exchange round = one replay of
a captured CUDA graph in the execution form the ensemble's autotuner keeps
(on GB300: 10 warp-tile sweep launches, the last also counting the unlike
bonds, then the exchange round).

  value      site-updates/s with the spins resident in HBM (CUDA events)
  e2e        the same through the C ABI with pinned host buffers: each step
             uploads every replica's int32 site values, runs the step and
             downloads them (the host<->device sync of a host AppLattice)
  plain_gpu  the same ensemble swept replica by replica with the plain
             per-colour phase kernel (a bounded sample, extrapolated)
  roofline   algorithmic HBM bytes (2 bytes per int8 site-update) / kernel
             time, against the measured copy bandwidth
  cpu_baseline  the reference's own colour sweep (SPPARKS built from its
             sources on this host) on one core over a bounded sample; the
             oracle port where the reference does not build

`--impl reference` times that CPU implementation alone on all host cores and
prints the same JSON line.

Usage: python bench.py [--gpus N] [--steps K] [--warmup W] [--impl ours|reference]
"""

from __future__ import annotations

import argparse
import json
import math
import os
import re
import statistics
import subprocess
import tempfile
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parent
sys.path.insert(0, str(ROOT))

METRIC = "site-updates/s on 1 GB300, batched vs plain GPU sweep; % of HBM roofline"
UNIT = "site-updates/s"
SEED = 56789
NREP = 512
SWEEPS_PER_STEP = 10
FULL_SWEEPS = 2000


def ensemble_config(seed=SEED, nrep=NREP):
    """Replica sizes and temperatures of the batched workload (seeded)."""
    rng = np.random.default_rng(seed)
    L = 32 * np.round(np.exp(rng.uniform(math.log(64), math.log(1024), nrep)) / 32).astype(np.int64)
    L = np.clip(L, 64, 1024).astype(np.int32)
    T = rng.uniform(1.5, 3.5, nrep)
    return L, T


def init_spins(L, seed=SEED):
    rng = np.random.default_rng(seed + 1)
    n = int(np.sum(L.astype(np.int64) ** 2))
    return (rng.integers(1, 3, n, dtype=np.int32)).astype(np.int32)


def measured_peaks():
    p = ROOT / "MEASURED_PEAKS.json"
    if p.exists():
        d = json.loads(p.read_text())
        return float(d["hbm_gbs"]), "measured"
    return 6800.0, "fallback"


def profile_traffic(name):
    """Per-launch DRAM traffic of kernel `name` from the committed ncu
    summaries (profiles/*.md, line `traffic_bytes_per_launch <name>: N`)."""
    for f in sorted((ROOT / "profiles").glob("*.md")):
        m = re.search(rf"traffic_bytes_per_launch {name}:\s*([0-9.eE+]+)", f.read_text())
        if m:
            return float(m.group(1)), f.name
    return None, None


def gpu_identity(device):
    """The benchmarked GPU as nvidia-smi names it: its UUID (or PCI bus id),
    taken from the CUDA device, so that CUDA_VISIBLE_DEVICES remapping cannot
    point the clock samples at another GPU.  Returns (id, how it was found)."""
    import torch

    props = torch.cuda.get_device_properties(device)
    cands = []
    uuid = getattr(props, "uuid", None)
    if uuid is not None:
        u = str(uuid)
        cands.append((u if u.startswith("GPU-") else "GPU-" + u, "uuid"))
    bus = getattr(props, "pci_bus_id", None)
    if bus is not None:
        cands.append((f"{getattr(props, 'pci_domain_id', 0):08x}:{bus:02x}:{getattr(props, 'pci_device_id', 0):02x}.0",
                      "pci bus id"))
    for ident, how in cands:
        try:
            r = subprocess.run(["nvidia-smi", f"--id={ident}", "--query-gpu=uuid", "--format=csv,noheader"],
                               capture_output=True, text=True, timeout=20)
            if r.returncode == 0 and r.stdout.strip():
                return ident, how
        except Exception:
            pass
    vis = os.environ.get("CUDA_VISIBLE_DEVICES", "")
    parts = [x.strip() for x in vis.split(",") if x.strip()]
    if parts and device < len(parts):
        return parts[device], "CUDA_VISIBLE_DEVICES entry"
    return str(device), "CUDA ordinal (no remapping in effect)"


class ClockSampler:
    """nvidia-smi clocks and throttle reasons during the timed region, on the
    benchmarked GPU named by identity (gpu_identity)."""

    Q = ("index,clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,"
         "clocks_event_reasons.hw_slowdown,clocks_event_reasons.hw_thermal_slowdown,"
         "clocks_event_reasons.sw_thermal_slowdown,clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.ident, self.ident_how = gpu_identity(device)
        self.proc = None
        self.path = Path(tempfile.gettempdir()) / f"spk_bench_clocks_{os.getpid()}.csv"

    def start(self):
        try:
            self.f = open(self.path, "w")
            self.proc = subprocess.Popen(["nvidia-smi", f"--id={self.ident}", f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "100"], stdout=self.f,
                                         stderr=subprocess.DEVNULL)
        except Exception:
            self.proc = None

    def stop(self):
        if not self.proc:
            return {"sm_mhz": None, "sm_max_mhz": None, "reasons": ["nvidia-smi unavailable"], "gpu": self.ident}
        self.proc.terminate()
        try:
            self.proc.wait(timeout=5)
        except Exception:
            self.proc.kill()
        self.f.close()
        sm, smax, reasons = [], [], set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for line in self.path.read_text().splitlines():
            p = [x.strip() for x in line.split(",")]
            if len(p) < 9:
                continue
            try:
                sm.append(float(p[1]))
                smax.append(float(p[2]))
            except ValueError:
                continue
            for k, nm in enumerate(names):
                if p[5 + k].lower().startswith("active"):
                    reasons.add(nm)
        try:
            self.path.unlink()
        except OSError:
            pass
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(smax) if smax else None,
                "reasons": sorted(reasons), "samples": len(sm), "gpu": self.ident, "gpu_id": self.ident_how}


# ---------------------------------------------------------------------------
# CPU implementations - reference arm and cpu_baseline
#
# The reference itself (kind "reference"): SPPARKS built from its own sources
# by oracle/ref/Makefile, natively on this host (from the staged copy of its
# sources where the reference tree is absent), driven through its library
# interface by oracle/_ref/runner_plain.  Each replica is one reference run:
# `app_style ising`, `lattice sq/4n`, `sweep color`, its temperature, its
# own seed, and `run 2` = 4 sweeps (dt_sweep = 1/2 for ising,
# src/app_ising.cpp:41); the runner times each `run` with a monotonic clock.
# The oracle port (kind "port", the C restatement) is the fallback when the
# reference did not build here.


def sample_replicas(nrep, procs, offset=0):
    """`nrep` random replicas of the workload's distribution, assigned to
    `procs` workers longest-first so that every worker holds about the same
    number of sites."""
    L, T = ensemble_config()
    rng = np.random.default_rng(7 + offset)
    pick = rng.choice(len(L), size=min(nrep, len(L)), replace=False)
    reps = sorted([(int(r), int(L[r]), float(T[r])) for r in pick], key=lambda x: -x[1])
    chunks, load = [[] for _ in range(procs)], [0] * procs
    for rep in reps:
        k = load.index(min(load))
        chunks[k].append(rep)
        load[k] += rep[1] ** 2
    return chunks


def _reference_script(reps, sweeps, warmup, steps, seed):
    lines = []
    for r, L, T in reps:
        lines += [f"seed {seed + r}", "app_style ising", "dimension 2", "lattice sq/4n 1.0",
                  f"region box block 0 {L} 0 {L} -0.5 0.5", "create_box box", "create_sites box",
                  "set site range 1 2", "sweep color", f"temperature {T!r}"]
        lines += [f"run {sweeps / 2!r}"] * warmup
        lines += [f"#! timed {k} run {sweeps / 2!r}" for k in range(steps)]
        lines.append("clear")
    return "\n".join(lines) + "\n"


def reference_cpu_rate(chunks, sweeps, warmup, steps, binary):
    """The reference's own colour sweep, one runner process per chunk, all
    at once.  A step is every replica of every chunk swept `sweeps` times;
    its time is the slowest worker's summed `run` time for that step.
    Returns (site-updates/s, updates, per-step seconds)."""
    procs, files = [], []
    tmpdir = Path(tempfile.mkdtemp(prefix="spk_ref_"))
    for w, reps in enumerate(chunks):
        f = tmpdir / f"in.{w}"
        f.write_text(_reference_script(reps, sweeps, warmup, steps, SEED))
        files.append(f)
        procs.append(subprocess.Popen([str(binary), str(f)], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                      text=True, cwd=str(tmpdir)))
    per_worker = []
    for pr in procs:
        out, err = pr.communicate()
        if pr.returncode != 0:
            raise RuntimeError(f"reference runner failed ({pr.returncode}): {err[-400:]}")
        t = [0.0] * steps
        for line in out.splitlines():
            p = line.split()
            if len(p) == 3 and p[0] == "timed":
                t[int(p[1])] += float(p[2])
        per_worker.append(t)
    for f in files:
        f.unlink()
    tmpdir.rmdir()
    step_s = [max(t[k] for t in per_worker) for k in range(steps)]
    updates = sum(L * L for reps in chunks for _, L, _ in reps) * sweeps * steps
    return updates / sum(step_s), updates, step_s


def _port_worker(args):
    reps, sweeps, seed = args
    import oracle

    done = 0
    t0 = time.perf_counter()
    for r, L, T in reps:
        cfg = oracle.make_cfg("sq/4n", L, L, 1, "ising", 2, T, seed=seed, stream_base=(r + 1) << 8)
        spin = oracle.init_spins(seed + r, L * L, 1, 2)
        oracle.color_sweeps(cfg, spin, 0, sweeps)
        done += L * L * sweeps
    return done, time.perf_counter() - t0


def port_cpu_rate(chunks, sweeps, pool=None):
    """Site-updates/s of the oracle port's colour sweep over `chunks` (wall
    time of the sample; `pool` is a persistent spawn pool of len(chunks))."""
    t0 = time.perf_counter()
    if pool is None:
        results = [_port_worker((c, sweeps, SEED)) for c in chunks]
    else:
        results = pool.map(_port_worker, [(c, sweeps, SEED) for c in chunks])
    wall = time.perf_counter() - t0
    updates = sum(r[0] for r in results)
    return updates / wall, updates, wall


def reference_binary():
    """runner_plain built natively here, or (None, why not)."""
    import oracle

    try:
        oracle.build_reference()
    except Exception as e:  # a failed native build falls back to the port
        return None, f"reference build failed: {str(e)[-200:]}"
    b = oracle.reference_binary("runner_plain")
    return (b, None) if b else (None, "reference sources absent on this host")


def run_reference(args):
    """The reference's CPU colour sweep on every host core: one reference
    runner per core, each step 4 random replicas per core (about equal sites
    per core) x 4 sweeps.  Falls back to the oracle port, labelled, when the
    reference cannot be built here."""
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    procs = os.cpu_count() or 1
    sweeps = 4
    binary, why = reference_binary()
    if binary:
        chunks = sample_replicas(4 * procs, procs)
        value, ups, step_s = reference_cpu_rate(chunks, sweeps, args.warmup, args.steps, binary)
        kind = "reference"
        sample = (f"{4 * procs} random replicas x {sweeps} sweeps per step, one reference runner per core: "
                  "SPPARKS built from its own sources on this host, app_style ising, sweep color, stock RandomPark")
    else:
        import multiprocessing as mp

        import oracle

        oracle.build()
        with mp.get_context("spawn").Pool(procs) as pool:
            for w in range(args.warmup):
                port_cpu_rate(sample_replicas(procs, procs, 1000 + w), 1, pool)
            step_s, ups = [], 0
            for k in range(args.steps):
                _, u, wall = port_cpu_rate(sample_replicas(4 * procs, procs, k), sweeps, pool)
                step_s.append(wall)
                ups += u
        value = ups / sum(step_s)
        kind = "port"
        sample = (f"{4 * procs} replicas x {sweeps} sweeps per step, oracle C restatement of "
                  f"AppIsing::site_event_rejection + colour sweep, one process per core ({why})")
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": args.gpus, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": 1000 * statistics.mean(step_s), "higher_is_better": True,
        "scaling": "weak", "vs_baseline": None, "dtype": "int32", "data": "synthetic",
        "impl": "reference",
        "config": {"workload": "batched 2D Ising ensemble, 512 sq/4n replicas L in [64,1024], kT in [1.5,3.5], "
                               "exchange every 10 sweeps", "step": f"{sweeps} sweeps of {4 * procs} random replicas, "
                                                                   "about equal sites per core",
                   "threads": procs},
        "cpu_baseline": {"value": value, "unit": UNIT, "cores": procs, "kind": kind, "sample": sample},
        "e2e": {"value": value, "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0},
    }
    print(json.dumps(line), flush=True)


def cpu_baseline_leg():
    """About 10 s of one host core on a bounded sample of the workload: the
    reference itself where it builds here, else the oracle port."""
    binary, why = reference_binary()
    if binary:
        chunks = sample_replicas(24, 1, 3)
        sweeps = 48  # about 1.6e8 site-updates: 8 s at the 2e7/s of one Grace core
        r, u, step_s = reference_cpu_rate(chunks, sweeps, 0, 1, binary)
        return {"value": r, "unit": UNIT, "cores": 1, "kind": "reference",
                "sample": f"24 random replicas x {sweeps} sweeps ({u:.3g} site-updates, {sum(step_s):.1f} s), "
                          "SPPARKS built from its own sources on this host (app_style ising, sweep color), 1 core"}
    import oracle

    oracle.build()
    r, u, w = port_cpu_rate(sample_replicas(48, 1, 0), 40)
    return {"value": r, "unit": UNIT, "cores": 1, "kind": "port",
            "sample": f"48 random replicas x 40 sweeps ({u:.3g} site-updates, {w:.1f} s), oracle C "
                      f"restatement of the reference colour sweep, 1 thread ({why})"}


# ---------------------------------------------------------------------------
# GPU arm


def max_over_ranks(value, dist, device="cpu"):
    """The timed region's length on the slowest rank (the job's time)."""
    if dist is None:
        return value
    import torch

    t = torch.tensor([float(value)], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def whole_job_rate(units_per_rank, world, job_ms):
    """Whole-job throughput: units all ranks processed / the job's time."""
    return units_per_rank * world / (job_ms * 1e-3)


def dist_setup(ngpus):
    if ngpus <= 1 or "RANK" not in os.environ:
        return 0, 1, None
    import torch
    import torch.distributed as dist

    rank = int(os.environ["RANK"])
    world = int(os.environ["WORLD_SIZE"])
    local = int(os.environ.get("LOCAL_RANK", rank))
    torch.cuda.set_device(local)
    dist.init_process_group("nccl")
    return rank, world, dist


def run_ours(args):
    import torch

    import spparks_gb300 as sg

    rank, world, dist = dist_setup(args.gpus)
    device = int(os.environ.get("LOCAL_RANK", "0")) if world > 1 else 0
    torch.cuda.set_device(device)

    def barrier():
        torch.cuda.synchronize()
        if dist:
            dist.barrier()

    # each rank runs its own ensemble (independent replicas; no collective)
    L, T = ensemble_config(seed=SEED + rank)
    spins = init_spins(L, seed=SEED + rank)
    nsites = int(np.sum(L.astype(np.int64) ** 2))
    ens = sg.Ensemble(L, T, "ising", 2, seed=SEED + rank, exchange_every=SWEEPS_PER_STEP, device=device)
    ens.upload(spins)
    ens_mode = ens.mode()  # the autotuner's choice of execution form, with its timings
    flush = torch.empty(256 << 20, dtype=torch.uint8, device=f"cuda:{device}")  # > 126 MB L2

    for _ in range(args.warmup):
        ens.run(SWEEPS_PER_STEP)
    ens.synchronize()

    # device-resident timed region: one graph replay per step, L2 flushed between steps
    launches0 = ens.launch_count()
    clocks = ClockSampler(device)
    clocks.start()
    barrier()
    step_ms = []
    kern_ms, kern_launches = 0.0, 0
    for _ in range(args.steps):
        flush.zero_()
        torch.cuda.synchronize()
        step_ms.append(ens.timed_run(SWEEPS_PER_STEP))
        k_ms, k_n = ens.sweep_kernel_ms()  # event nodes around the sweep kernels in the replayed graph
        kern_ms += k_ms
        kern_launches += k_n
    barrier()
    clk = clocks.stop()
    launches = ens.launch_count() - launches0
    st = ens.stats()
    total_ms = max_over_ranks(sum(step_ms), dist, f"cuda:{device}")
    updates_rank = nsites * SWEEPS_PER_STEP * args.steps
    value = whole_job_rate(updates_rank, world, total_ms)
    ms_step = total_ms / args.steps

    # end to end through the C ABI with pinned host buffers
    host_in = torch.from_numpy(spins).pin_memory()
    host_out = torch.empty_like(host_in).pin_memory()
    ein, eout = host_in.numpy(), host_out.numpy()
    # pipelined: the whole job of the workload (2000 sweeps = 200 steps, or
    # the timed steps if more), so the pipeline's fill and drain weigh as
    # they do in a real run
    e2e_steps = max(args.steps, FULL_SWEEPS // SWEEPS_PER_STEP)
    seq_steps = max(1, min(args.steps, 20))  # one call after another: a sample
    # pipelined (spkgpu_ensemble_run_io: a step's input and the previous
    # step's result cross the host link while the sweeps run), then the same
    # steps one call after another (upload, run, download)
    barrier()
    t0 = time.perf_counter()
    for _ in range(e2e_steps):
        ens.run_io(ein, eout, SWEEPS_PER_STEP)
    ens.synchronize()
    barrier()
    e2e_ms = max_over_ranks((time.perf_counter() - t0) * 1e3, dist, f"cuda:{device}")
    e2e_value = whole_job_rate(nsites * SWEEPS_PER_STEP * e2e_steps, world, e2e_ms)
    barrier()
    t0 = time.perf_counter()
    for _ in range(seq_steps):
        ens.upload(ein)
        ens.run(SWEEPS_PER_STEP)
        ens.download(eout)
    barrier()
    seq_ms = max_over_ranks((time.perf_counter() - t0) * 1e3, dist, f"cuda:{device}")
    e2e_seq_value = whole_job_rate(nsites * SWEEPS_PER_STEP * seq_steps, world, seq_ms)

    # plain GPU sweeps: the same replicas one lattice at a time (a sample of
    # replicas, 10 sweeps each, extrapolated by sites), once with the generic
    # per-colour phase kernel and once with the repo's fastest single-lattice
    # sweep (the fused warp-tile kernel of spkgpu_sweep): batched over the
    # latter measures what batching gains, over the former the kernel too
    rng = np.random.default_rng(11)
    pick = rng.choice(len(L), size=48, replace=False)
    plain = {}
    for variant in (1, 0):
        plain_ms, plain_sites = 0.0, 0
        for r in pick:
            lat = sg.Lattice("sq/4n", int(L[r]), int(L[r]), 1, "ising", 2, spin_bytes=1, seed=SEED, variant=variant)
            lat.set_temperature(float(T[r]))
            lat.upload(ens.replica(spins, r))
            lat.timed_sweeps(2)
            plain_ms += lat.timed_sweeps(SWEEPS_PER_STEP)
            plain_sites += int(L[r]) ** 2 * SWEEPS_PER_STEP
            lat.close()
        plain[variant] = plain_sites / (plain_ms * 1e-3)
    plain_rate, plain_fused = plain[1], plain[0]

    peak, peak_kind = measured_peaks()
    # dominant kernel: the persistent kernel (all sweeps of a step) or the
    # per-sweep launch; int8 sites, one read and one write per update
    persistent = ens_mode["mode"] == "persistent"
    kname = ("ensemble_kernel" if persistent else
             "ensemble_warp_kernel" if ens_mode["mode"] == "warps" else "ensemble_sweep_kernel")
    alg_bytes = 2.0 * 1.0 * nsites * (SWEEPS_PER_STEP if persistent else 1)
    kernel_ms = kern_ms / max(kern_launches, 1)
    achieved = alg_bytes / (kernel_ms * 1e-3) / 1e9
    traffic, traffic_src = profile_traffic(kname)
    # the draw-side ceiling: one Philox4x32-10 block per four Ising sites
    philox_bps = sg.philox_rate(device, 1024)

    if rank != 0:
        return
    configs = measure_configs(sg, peak, peak_kind)
    cpu = None if args.no_cpu else cpu_baseline_leg()
    if not args.no_cpu:
        ref_cfg = reference_cpu_configs()
        for name in ("C0", "C1", "C4"):
            configs[name]["cpu_baseline"] = ref_cfg[name]
        configs["C3_serial"]["cpu_baseline"] = ref_cfg["C3"]
    line = {
        "metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": args.steps,
        "warmup": args.warmup, "ms_per_step": ms_step, "higher_is_better": True, "scaling": "weak",
        "vs_baseline": None, "dtype": "int8", "data": "synthetic (seeded replicas, uniform spins)",
        "config": {"workload": "batched 2D Ising ensemble: 512 sq/4n replicas, L log-uniform in [64,1024] "
                               "rounded to 32, kT uniform [1.5,3.5], exchange every 10 sweeps",
                   "replicas": int(len(L)), "sites": nsites, "sweeps_per_step": SWEEPS_PER_STEP,
                   "full_job_sweeps": FULL_SWEEPS, "l2": "flushed between steps (256 MiB memset)",
                   "parallelism": f"replicas, {world} independent ensemble(s)",
                   "execution": ens_mode},
        "e2e": {"value": e2e_value, "unit": UNIT, "h2d_bytes_per_step": int(nsites * 4),
                "d2h_bytes_per_step": int(nsites * 4), "steps": e2e_steps,
                "api": "spkgpu_ensemble_run_io (pinned int32 host buffers, steps pipelined, the whole 2000-sweep job)",
                "sequential": {"value": e2e_seq_value, "steps": seq_steps,
                               "api": "spkgpu_ensemble_upload + run + download per step"}},
        "gpu_launches": int(launches),
        "plain_gpu": {"value": plain_rate, "unit": UNIT, "sample": "48 replicas x 10 sweeps, per-colour "
                      "phase kernel, one lattice at a time", "batched_over_plain": value / world / plain_rate,
                      "fused": {"value": plain_fused, "unit": UNIT,
                                "sample": "the same 48 replicas x 10 sweeps, fused warp-tile sweep (spkgpu_sweep), "
                                          "one lattice at a time", "batched_over_plain": value / world / plain_fused}},
        "roofline": {"bound": "hbm", "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
                     "peak_kind": f"{peak_kind} copy bandwidth (burst)", "traffic": traffic,
                     "traffic_source": traffic_src,
                     "alg_bytes_per_launch": alg_bytes, "kernel_ms_per_launch": kernel_ms,
                     "kernel": kname + (" (one launch per step of 10 sweeps + exchange)" if persistent
                                        else " (one launch per sweep)")},
        "rng_ceiling": {"philox_blocks_per_s": philox_bps, "site_updates_per_s": 4.0 * philox_bps,
                        "frac": value / world / (4.0 * philox_bps),
                        "source": "spkgpu_philox_rate: the sweeps' Philox code alone, 4 Ising sites per block"},
        "cpu_baseline": cpu,
        "configs": configs,
        "clocks": clk,
        "exchange": {"tries": st["exchange_tries"], "accepts": st["exchange_accepts"]},
    }
    print(json.dumps(line), flush=True)


# ---------------------------------------------------------------------------
# The other configurations: each timed on the GPU (CUDA events on the
# lattice's stream, or the host clock around a synchronous KMC run) and, on
# one host core each, the reference itself on a bounded sample (run side by
# side, one process per configuration).

# (label, lattice, n, app, nspins, spin bytes, kT): the single-lattice sweeps
C0 = ("sq/4n", (128, 128, 1), "ising", 2, 4, 2.269)
C1 = ("sc/26n", (256, 256, 256), "potts/neighonly", 100, 2, 0.5)
C4 = ("sc/6n", (1536, 1536, 1536), "ising", 2, -1, 4.5115)
BYTES_PER_UPDATE = {4: 8.0, 2: 4.0, 1: 2.0, -1: 0.25}  # 2 s per site-update, s = storage bytes


def _reference_lines(lattice, n, app, q, T, tail):
    nx, ny, nz = n
    dim = 3 if lattice.startswith("sc") else 2
    zr = f"0 {nz}" if dim == 3 else "-0.5 0.5"
    app_line = "app_style ising" if app == "ising" else f"app_style {app} {q}"
    return [f"seed {SEED}", app_line, f"dimension {dim}", f"lattice {lattice} 1.0",
            f"region box block 0 {nx} 0 {ny} {zr}", "create_box box", "create_sites box",
            f"set site range 1 {q}"] + tail


REF_CPU_CASES = {
    # 100 sweeps of 128^2, 40 times (dt_sweep = 1/2 for ising)
    "C0": dict(lines=_reference_lines("sq/4n", (128, 128, 1), "ising", 2, 2.269,
                                      ["sweep color", "temperature 2.269"] +
                                      [f"#! timed {k} run 50" for k in range(40)]),
               updates=128 * 128 * 100 * 40, sample="128^2 sq/4n ising kT 2.269, 40 x 100 sweeps"),
    # 96^3 sc/26n potts/neighonly Q=100: 12 sweeps (dt_sweep = 1/26; the run stops half a sweep early)
    "C1": dict(lines=_reference_lines("sc/26n", (96, 96, 96), "potts/neighonly", 100, 0.5,
                                      ["sweep color", "temperature 0.5", f"#! timed 0 run {11.5 / 26!r}"]),
               updates=96 ** 3 * 12, sample="96^3 sc/26n potts/neighonly Q=100 kT 0.5, 12 sweeps"),
    # 2048^2 sq/8n potts Q=50, solve_style tree with sector yes, serial: events to t = 0.03
    "C3": dict(lines=_reference_lines("sq/8n", (2048, 2048, 1), "potts", 50, 1.0,
                                      ["solve_style tree", "sector yes", "temperature 1.0", "#! timed 0 run 0.03",
                                       "#! appstats"]),
               updates=None, sample="2048^2 sq/8n potts Q=50 kT 1, tree, 4 sectors, one processor, to t = 0.03"),
    # 128^3 sc/6n ising (the full 1536^3 lattice does not fit a CPU run): 16 sweeps
    "C4": dict(lines=_reference_lines("sc/6n", (128, 128, 128), "ising", 2, 4.5115,
                                      ["sweep color", "temperature 4.5115", "#! timed 0 run 8"]),
               updates=128 ** 3 * 16, sample="128^3 sc/6n ising kT 4.5115, 16 sweeps"),
}


def reference_cpu_configs():
    """The reference on one host core per configuration, all at once."""
    binary, why = reference_binary()
    if not binary:
        return {k: {"unavailable": why} for k in REF_CPU_CASES}
    tmpdir = Path(tempfile.mkdtemp(prefix="spk_refcfg_"))
    procs = {}
    for name, case in REF_CPU_CASES.items():
        f = tmpdir / f"in.{name}"
        f.write_text("\n".join(case["lines"]) + "\n")
        procs[name] = subprocess.Popen([str(binary), str(f)], stdout=subprocess.PIPE, stderr=subprocess.PIPE,
                                       text=True, cwd=str(tmpdir))
    out = {}
    for name, pr in procs.items():
        o, e = pr.communicate()
        case = REF_CPU_CASES[name]
        if pr.returncode != 0:
            out[name] = {"unavailable": f"reference run failed: {e[-200:]}"}
            continue
        secs = sum(float(l.split()[2]) for l in o.splitlines() if l.startswith("timed "))
        if case["updates"] is None:  # KMC: events from the app's own stats line
            st = [l.split() for l in o.splitlines() if l.startswith("appstats ")][-1]
            units, unit = int(st[2]), "events/s"
        else:
            units, unit = case["updates"], UNIT
        out[name] = {"value": units / secs, "unit": unit, "cores": 1, "kind": "reference",
                     "sample": f"{case['sample']} ({units:.3g} in {secs:.1f} s), SPPARKS built from its own sources "
                               "on this host, stock RandomPark"}
        (tmpdir / f"in.{name}").unlink()
    tmpdir.rmdir()
    return out


def _sweep_rate(sg, cfg, nsweeps, warm=1, seed=SEED, variant=0):
    lattice, n, app, q, sb, T = cfg
    lat = sg.Lattice(lattice, *n, app, q, spin_bytes=sb, seed=seed, variant=variant)
    lat.set_temperature(T)
    lat.init_spins(1, q)
    lat.timed_sweeps(warm)
    ms = lat.timed_sweeps(nsweeps)
    sites = lat.n
    launches = lat.launch_count()
    lat.close()
    return sites * nsweeps / (ms * 1e-3), ms / nsweeps, launches


def _roofline(rate, bytes_per_update, peak, peak_kind, bound="hbm"):
    achieved = rate * bytes_per_update / 1e9
    return {"bound": bound, "achieved": achieved, "peak": peak, "unit": "GB/s", "frac": achieved / peak,
            "peak_kind": f"{peak_kind} copy bandwidth", "bytes_per_update": bytes_per_update}


def measure_configs(sg, peak, peak_kind):
    """GPU rates of C0, C1, C3 (serial and processor grid) and C4 (bit-packed
    and int8 on the same lattice), each on its own stream."""
    res = {}
    r, ms, _ = _sweep_rate(sg, C0, 100, warm=5)
    res["C0"] = {"workload": "128^2 sq/4n ising int32 kT 2.269, 100 sweeps (the whole job)", "value": r,
                 "unit": UNIT, "ms_per_sweep": ms,
                 "roofline": {**_roofline(r, 8.0, peak, peak_kind, "latency"),
                              "note": "64 KB lattice held in one 8-CTA cluster's shared memory for all 100 sweeps "
                                      "(one launch); two cluster barriers per sweep bound it, not HBM"}}
    r, ms, _ = _sweep_rate(sg, C1, 20, warm=2)
    res["C1"] = {"workload": "256^3 sc/26n potts/neighonly Q=100 int16 kT 0.5, 20 of the 1000 sweeps", "value": r,
                 "unit": UNIT, "ms_per_sweep": ms, "roofline": _roofline(r, 4.0, peak, peak_kind, "alu")}
    rp, msp, _ = _sweep_rate(sg, C4, 5)
    r8, ms8, _ = _sweep_rate(sg, C4[:4] + (1,) + C4[5:], 2)
    res["C4"] = {"workload": "1536^3 sc/6n ising kT 4.5115 (3.6e9 sites), 5 of the 500 sweeps", "value": rp,
                 "unit": UNIT, "ms_per_sweep": msp, "roofline": _roofline(rp, 0.25, peak, peak_kind, "alu"),
                 "int8_same_lattice": {"value": r8, "unit": UNIT, "ms_per_sweep": ms8,
                                       "roofline": _roofline(r8, 2.0, peak, peak_kind),
                                       "kernel": "per-colour phase kernel, int8"},
                 "packed_over_int8": rp / r8}
    res.update(measure_configs_c3(sg))
    lat = sg.Lattice("sq/8n", 2048, 2048, 1, "potts", 50, spin_bytes=4, nsector=4, procs=(32, 32, 1), seed=SEED)
    lat.set_temperature(1.0)
    lat.init_spins(1, 50)
    lat.kmc_setup(fp64=False)
    st = lat.kmc_run(0.0, 0.2)
    lat.close()
    res["C3_grid"]["fp32_propensities"] = {"prop_rel_err": st["prop_rel_err"], "dt_rel_err": st["dt_rel_err"],
                                           "events": st["naccept"], "t": st["time"],
                                           "against": "all-FP64 propensities of the same chains"}
    return res


def measure_configs_c3(sg, serial_t=0.02):
    """Tree KMC on 2048^2 sq/8n Potts Q=50: serial (the configuration as
    written) and on a 32x32 processor grid, events/s (host clock around a
    synchronous run, after a short warm-up pass)."""
    res = {}
    for name, procs, tend, fp64 in (("C3_serial", (1, 1, 1), serial_t, True), ("C3_grid", (32, 32, 1), 1.0, True),
                                    ("C3_serial_fp32", (1, 1, 1), serial_t, False)):
        lat = sg.Lattice("sq/8n", 2048, 2048, 1, "potts", 50, spin_bytes=4, nsector=4, procs=procs, seed=SEED)
        lat.set_temperature(1.0)
        lat.init_spins(1, 50)
        lat.kmc_setup(fp64=fp64)
        w = lat.kmc_run(0.0, 1e-4)  # warm-up: one short pass (tree build, first kernels)
        t0 = time.perf_counter()
        st = lat.kmc_run(w["time"], w["time"] + tend)
        wall = time.perf_counter() - t0
        ev = st["naccept"] - w["naccept"]
        lat.close()
        res[name] = {"workload": f"2048^2 sq/8n potts Q=50 kT 1, tree KMC, 4 sectors, processors "
                                 f"{procs[0]}x{procs[1]}, {'FP64' if fp64 else 'FP32 (FP64 tree and clock)'} "
                                 f"propensities, t += {tend}",
                     "value": ev / wall, "unit": "events/s", "events": ev, "passes": st["npass"],
                     "roofline": {"bound": "latency", "frac": None,
                                  "note": "a chain of dependent events per sector; the HBM fraction is not meaningful"}}
        if not fp64:
            res[name]["errors"] = {"prop_rel_err": st["prop_rel_err"], "dt_rel_err": st["dt_rel_err"],
                                   "against": "all-FP64 propensities of the same chains"}
    return res


def kernel_case(name):
    """Small fixed workloads that launch one hot kernel each, for profilers
    (the commands in profiles/*.md); prints a one-line status."""
    import spparks_gb300 as sg

    if name == "ensemble":  # 160 uneven replicas, 1.06e8 sites (2 x 106 MB > L2): two launches of 10 sweeps
        L = [1024, 768, 512, 1024, 896, 256, 1024, 640] * 20
        T = list(np.linspace(1.5, 3.5, len(L)))
        rng = np.random.default_rng(3)
        ens = sg.Ensemble(L, T, "ising", 2, seed=3, exchange_every=10)
        ens.upload(rng.integers(1, 3, sum(l * l for l in L)).astype(np.int32))
        ens.run(10)
        ens.run(10)
        print("ensemble", ens.stats())
    elif name == "fused":  # 12288^2 int8 Ising (2 x 151 MB > L2), fused tile sweeps
        lat = sg.Lattice("sq/4n", 12288, 12288, 1, "ising", 2, spin_bytes=1, seed=5)
        lat.set_temperature(2.269)
        lat.init_spins(1, 2)
        lat.sweep(5)
        print("fused", lat.stats())
    elif name == "rows":  # potts/neighonly Q=100 sc/26n 256x256x128 int16, row-pair sweeps
        lat = sg.Lattice("sc/26n", 256, 256, 128, "potts/neighonly", 100, spin_bytes=2, seed=5)
        lat.set_temperature(0.5)
        lat.init_spins(1, 100)
        lat.sweep(2)
        print("rows", lat.stats())
    elif name == "c0":  # sq/4n Ising 128^2 int32, 100 sweeps in one call (the cluster-resident sweep)
        lat = sg.Lattice("sq/4n", 128, 128, 1, "ising", 2, spin_bytes=4, seed=5)
        lat.set_temperature(2.269)
        lat.init_spins(1, 2)
        lat.sweep(100)
        lat.sweep(100)
        print("c0", lat.stats())
    elif name == "packed":  # bit-packed Ising sc/6n 512^3
        lat = sg.Lattice("sc/6n", 512, 512, 512, "ising", 2, spin_bytes=-1, seed=5)
        lat.set_temperature(4.5115)
        lat.init_spins(1, 2)
        lat.sweep(2)
        print("packed", lat.stats())
    elif name == "rates":  # site-updates/s of the single-lattice sweeps, CUDA events on each lattice's stream
        cases = [
            ("sq/4n 128^2 ising int32, 100 sweeps", ("sq/4n", 128, 128, 1, "ising", 2, 4), 2.269, 100),
            ("sc/26n 256^3 potts/neighonly Q=100 int16", ("sc/26n", 256, 256, 256, "potts/neighonly", 100, 2), 0.5, 5),
            ("sc/6n 1536^3 ising bit-packed", ("sc/6n", 1536, 1536, 1536, "ising", 2, -1), 4.5115, 3),
            ("sc/6n 1536^3 ising int8", ("sc/6n", 1536, 1536, 1536, "ising", 2, 1), 4.5115, 2),
            ("sq/4n 12288^2 ising int8", ("sq/4n", 12288, 12288, 1, "ising", 2, 1), 2.269, 20),
            ("sq/4n 12288^2 ising int16", ("sq/4n", 12288, 12288, 1, "ising", 2, 2), 2.269, 10),
            ("sq/4n 12288^2 potts Q=2 int8", ("sq/4n", 12288, 12288, 1, "potts", 2, 1), 1.0, 10),
        ]
        for label, (lt, nx, ny, nz, app, q, sb), temp, nsw in cases:
            lat = sg.Lattice(lt, nx, ny, nz, app, q, spin_bytes=sb, seed=56789)
            lat.set_temperature(temp)
            lat.init_spins(1, q)
            lat.timed_sweeps(1)
            ms = lat.timed_sweeps(nsw)
            print(f"{label}: {ms / nsw:.4f} ms per sweep, {lat.n * nsw / (ms * 1e-3):.3e} site-updates/s", flush=True)
            lat.close()
    elif name == "c3":  # events/s of tree KMC on the 2048^2 configuration, serial and on the 32x32 grid
        res = measure_configs_c3(sg)
        for k, v in res.items():
            print(k, f"{v['value']:.4g} events/s", v["events"], "events", v["passes"], "passes", flush=True)
    elif name == "kmc_serial":  # tree KMC Potts Q=50 sq/8n 1024^2, one processor, 4 sectors, a short run
        lat = sg.Lattice("sq/8n", 1024, 1024, 1, "potts", 50, spin_bytes=4, nsector=4, seed=5)
        lat.set_temperature(1.0)
        lat.init_spins(1, 50)
        lat.kmc_setup(fp64=True)
        print("kmc_serial", lat.kmc_run(0.0, 0.005))
    elif name == "kmc":  # tree KMC Potts Q=50 sq/8n 1024^2, 32x32 processor grid, 4 sectors
        lat = sg.Lattice("sq/8n", 1024, 1024, 1, "potts", 50, spin_bytes=4, nsector=4, procs=(32, 32, 1), seed=5)
        lat.set_temperature(1.0)
        lat.init_spins(1, 50)
        lat.kmc_setup(fp64=True)
        print("kmc", lat.kmc_run(0.0, 0.3))
    else:
        raise SystemExit(f"unknown kernel case {name}")


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=200)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", choices=["ours", "reference"], default="ours")
    ap.add_argument("--no-cpu", action="store_true", help="skip the CPU baseline sample")
    ap.add_argument("--kernel-case", choices=["ensemble", "fused", "rows", "c0", "packed", "kmc", "kmc_serial", "rates",
                                              "c3"],
                    help="run one small profiling workload instead of the benchmark")
    args = ap.parse_args()
    if args.kernel_case:
        kernel_case(args.kernel_case)
        return
    if args.warmup < 3:
        args.warmup = 3
    if args.impl == "reference":
        run_reference(args)
    else:
        run_ours(args)


if __name__ == "__main__":
    main()
