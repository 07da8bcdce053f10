#!/usr/bin/env python3
"""Throughput benchmark: aggregate Langevin steps/s of batched replicas.

Workload (the batched configuration of the benchmark description): 64 replicas of
a seeded 346-nt synthetic TIS chain (1037 beads) in a 350 A box, Mg2+ swept
0..20 mM in 64 linear steps at 76 mM KCl (ion numbers by the reference's rule,
4.6k-6.2k particles per replica), T = 298 K (0.59219 kcal/mol), h = 0.05,
Coulomb cutoff 30 A, SR list radius 12+3 A, LR refresh every 10 steps,
independent seeds.  Mixed precision (FP32 pair/bonded math, int64 fixed-point
forces, FP64 integration), all replicas advanced together by one CUDA graph.

A "step" advances every replica by one Langevin step; value = replica-steps/s
over all GPUs.  Inputs (the systems) are synthetic and generated here.

  python bench.py [--gpus N] [--steps K] [--warmup W] [--impl gpu|reference]

--impl reference times the reference's own CPU engine (oracle/_ref/tis_ref_bench,
built -O3 from the reference sources; else the C oracle port) on the host cores,
one replica per core, on a bounded sample of the same workload.

Besides the headline line's fields, the GPU arm reports the plain single-replica
FP64 GPU path on the central system (the batching denominator), kernel times
inside the replayed step, an end-to-end number through the C ABI over the same
steps, the reference engine on the host cores, and the other configurations of
the benchmark description: the 76-nt system in FP64 (GPU and one host core), the
central single replica, the parameter gradient over 10^4 frames and through
200-step trajectories, and the large system.
"""
import argparse
import json
import os
import subprocess
import sys
import tempfile
import threading
import time
from concurrent.futures import ThreadPoolExecutor

# each replica group's graph runs on its own streams; enough hardware work queues
# keep queued graphs of different groups from waiting on one another
os.environ.setdefault("CUDA_DEVICE_MAX_CONNECTIONS", "32")

ROOT = os.path.dirname(os.path.abspath(__file__))
sys.path.insert(0, os.path.join(ROOT, "16s-central-folding_gb300"))
sys.path.insert(0, os.path.join(ROOT, "oracle"))
sys.path.insert(0, os.path.join(ROOT, "tests"))

N_REPLICAS = 64
N_NT = 346
BOX = 350.0
RC = 30.0
T_298 = 0.59219
GEN_SEED = 2000
METRIC = "aggregate Langevin steps/s, batched mixed-prec vs plain GPU, force rel-err <=1e-5"
UNIT = "replica-steps/s"
GRAPH_STEPS = 100
# Untimed steps between the first list build and the warm-up: the build makes every
# replica's lists fresh at once, so their next rebuilds (every ~33 steps) come in
# bursts for the first hundred or so steps; after these steps they are spread out as
# in a long run, and a short timed window measures the run's steady state.
EQUIL_STEPS = 1000


def replica_specs(n=N_REPLICAS):
    from tis_gb300 import synth
    ions = synth.batch_mg_sweep(n_replicas=n, mg_max_mm=20.0, kcl_mm=76.0, box=BOX, n_nt=N_NT)
    return [dict(n_mg=m, n_cl=c, n_k=k, seed=1000 + r) for r, (m, c, k) in enumerate(ions)]


def rank_replica_specs(rank, n=N_REPLICAS):
    """The batch of one rank: replicas only, so every rank runs the whole workload
    with its own seeds (offset by 100000 x rank) and nothing is exchanged."""
    specs = replica_specs(n)
    for sp in specs:
        sp["seed"] += 100000 * rank
    return specs


def max_over_ranks(ms, world, device=None):
    """The slowest rank's timed region in ms (the job ends with it); the one
    collective of a multi-rank run, outside the timed region."""
    if world <= 1:
        return ms
    import torch
    import torch.distributed as dist
    t = torch.tensor([ms], dtype=torch.float64, device=device)
    dist.all_reduce(t, op=dist.ReduceOp.MAX)
    return float(t.item())


def job_value(ms, world, n_rep, steps):
    """Whole-job replica-steps/s: every rank's replicas over the slowest rank's time."""
    return world * n_rep * steps / (ms / 1000.0)


def make_inputs(tmp):
    from tis_gb300 import synth
    return synth.generate(tmp, "central", N_NT, seed=GEN_SEED, n_hb_pairs=120)


def load_systems(files, specs):
    from tis_gb300 import System

    def one(sp):
        return System.load(files["pdb"], files["bonds"], files["stacks"], files["maxikey"], T=T_298, box=BOX, rc=RC,
                           center=500, rng=1, **sp)

    with ThreadPoolExecutor(max_workers=min(16, os.cpu_count() or 4)) as ex:
        return list(ex.map(one, specs))


class ClockSampler:
    """Samples SM clocks and throttle reasons with nvidia-smi during the timed region."""

    Q = ("clocks.sm,clocks.max.sm,power.draw,clocks_event_reasons.active,clocks_event_reasons.hw_slowdown,"
         "clocks_event_reasons.hw_thermal_slowdown,clocks_event_reasons.sw_thermal_slowdown,"
         "clocks_event_reasons.sw_power_cap")

    def __init__(self, device=0):
        self.rows, self.proc, self.device = [], None, device

    def __enter__(self):
        try:
            self.proc = subprocess.Popen(["nvidia-smi", "-i", str(self.device), f"--query-gpu={self.Q}",
                                          "--format=csv,noheader,nounits", "-lms", "200"],
                                         stdout=subprocess.PIPE, stderr=subprocess.DEVNULL, text=True)
            self.th = threading.Thread(target=self._read, daemon=True)
            self.th.start()
        except OSError:
            self.proc = None
        return self

    def _read(self):
        for line in self.proc.stdout:
            self.rows.append([v.strip() for v in line.split(",")])

    def __exit__(self, *a):
        if self.proc:
            self.proc.terminate()
            try:
                self.proc.wait(timeout=5)
            except subprocess.TimeoutExpired:
                self.proc.kill()

    def summary(self):
        import statistics
        sm = [float(r[0]) for r in self.rows if len(r) >= 8 and r[0].replace(".", "").isdigit()]
        mx = [float(r[1]) for r in self.rows if len(r) >= 8 and r[1].replace(".", "").isdigit()]
        reasons = set()
        names = ["hw_slowdown", "hw_thermal_slowdown", "sw_thermal_slowdown", "sw_power_cap"]
        for r in self.rows:
            if len(r) >= 8:
                for n, v in zip(names, r[4:8]):
                    if v.lower() == "active":
                        reasons.add(n)
        return {"sm_mhz": statistics.median(sm) if sm else None, "sm_max_mhz": max(mx) if mx else None,
                "reasons": sorted(reasons), "samples": len(self.rows)}


def fp32_roofline(device, clocks, entries_per_launch, launch_ms):
    """The SR pair kernel against the FP32 roofline: its algorithmic FLOPs per launch
    (FLOP_PER_SR_ENTRY per list entry) over its in-step duration, and the GPU's FP32
    peak at the SM clock sampled during the timed region (SMs x 128 lanes x 2)."""
    import torch
    sms = torch.cuda.get_device_properties(device).multi_processor_count
    mhz = (clocks or {}).get("sm_mhz") or 2070.0
    peak = sms * 128 * 2 * mhz * 1e6 / 1e12
    flops = FLOP_PER_SR_ENTRY * entries_per_launch
    ach = flops / (launch_ms * 1e-3) / 1e12 if launch_ms > 0 else None
    return {"kernel": "pair_sr", "alg_flops_per_launch": flops, "achieved_tflops": ach, "peak_tflops": peak,
            "unit": "TFLOP/s", "frac": ach / peak if ach is not None else None,
            "ncu_fma_pipe_frac": NCU_FMA_PIPE.get("pair_sr"),
            "model": f"{FLOP_PER_SR_ENTRY} FLOP per SR list entry; peak at the sampled SM clock"}


def measured_peaks():
    try:
        with open(os.path.join(ROOT, "MEASURED_PEAKS.json")) as f:
            d = json.load(f)
        return d["hbm_gbs"], "measured"
    except Exception:
        return 6800.0, "fallback"


# Algorithmic (compulsory) HBM bytes of each stage per step of the whole batch:
# every array the stage must read or write once, gathers through cache not counted
# again.  n: particles; sr, lr: mean SR / LR neighbours per particle; lr_frac: share
# of particles whose LR sum is refreshed in a step; nreb: particles of the replicas
# that rebuild in a step; nrna: RNA beads; items: bonded terms + stacks; nhb: H-bond
# candidates (all summed over the replicas).
#   pair_sr:   q (16) + count (4) + list (4 sr) + force sum read-modify-write (48)
#   pair_lr:   (q 16 + count 4 + list 4 lr + LR force store 24) x lr_frac
#   bonded:    index/parameter record per item (32) + force RMW per RNA bead (48) + its q (16)
#   hbond:     per candidate index/natives record (96) + its six beads' q (96) and force
#              RMW (288); the step's 3000 Gaussians per replica (8 each)
#   shift:     per replica the centre bead's state (about 200)
#   integrate: read x, x_old, v (72), force sums (48), q (16); write x, x_old, v (72),
#              zeroed force sum (24), q (16): 248
#   cells:     per rebuilt particle x, y, z, q (40), cell id (4, written and read), slot
#              (4, written and read), cell-ordered copy of q (16 written)
#   search:    per rebuilt particle its cell-ordered q (16), cell id (4), the list
#              entries written (4 (sr + lr)) and counts (8)
def stage_bytes(n, sr, lr, lr_frac, nreb, nrna, items, nhb, nrep):
    return {
        "pair_sr": (16 + 4 + 4 * sr + 48) * n,
        "pair_lr": (16 + 4 + 4 * lr + 24) * n * lr_frac,
        "bonded": 32 * items + (48 + 16) * nrna,
        "hbond": (96 + 96 + 288) * nhb + 3000 * 8 * nrep,
        "shift": 200 * nrep,
        "integrate": 248 * n,
        "cells": (40 + 8 + 8 + 16) * nreb,
        "search": (16 + 4 + 4 * (sr + lr) + 8) * nreb,
    }


# DRAM bytes per replica of each step kernel's launch: dram__bytes_read.sum +
# dram__bytes_write.sum of one launch over a group of 8 replicas (about 43k
# particles; cold L2, serialised) divided by 8, from ncu captures of
# `python bench.py --steps 40 --warmup 3 --no-extras --groups 8` with --clock-control
# none, --kernel-name-base mangled and -k set to the kernel (None: no capture of a
# stepping launch).  Scaled to the batch by the number of replicas.
NCU_DRAM_BYTES_PER_REPLICA = {"pair_sr": 3.04e6 / 8, "pair_lr": None, "bonded": 1.24e6 / 8, "hbond": 0.479e6 / 8,
                              "shift": 0.04e6 / 8, "integrate": 5.35e6 / 8, "cells": 0.03e6 / 8, "search": None}


# Algorithmic FP32 work of the SR pair kernel per list entry evaluated: the distance
# from the integer differences (3 conversions folded into 3 mul, 2 fma: 8), the LJ or
# the Coulomb term (about 12: square root, reciprocal powers or the screened form),
# and the force accumulation (6).
FLOP_PER_SR_ENTRY = 26


# FP32 (FMA) pipe and issue-slot use of each kernel from its committed ncu capture
# (`--set full`, one launch over a group of 8 replicas; profiles/ncu_full_*.md):
# sm__pipe_fma_cycles_active and smsp__issue_active as fractions of their peaks.
NCU_FMA_PIPE = {"pair_sr": 0.0371, "hbond": 0.0621, "search": 0.0526, "bonded": 0.0632}
NCU_ISSUE_ACTIVE = {"pair_sr": 0.1469, "hbond": 0.1379, "search": 0.1452, "bonded": 0.1523}


def cpu_sample(files, specs, steps, workers):
    """Reference CPU engine on `workers` replicas in parallel, `steps` steps each."""
    import build_ref
    exe = build_ref.build(bench=True)
    kind = "reference" if exe else "port"
    sample = specs[:: max(1, len(specs) // workers)][:workers]

    def run_ref(sp):
        args = [exe, "--pdb", files["pdb"], "--bonds", files["bonds"], "--stacks", files["stacks"],
                "--maxikey", files["maxikey"], "--box", str(BOX), "--rc", str(RC), "--T", str(T_298),
                "--nMg", str(sp["n_mg"]), "--nCl", str(sp["n_cl"]), "--nK", str(sp["n_k"]),
                "--seed", str(sp["seed"]), "--center", "500", "--steps", str(steps), "--time"]
        out = subprocess.run(args, check=True, capture_output=True, text=True).stdout
        return json.loads(out.strip().splitlines()[-1])["seconds"]

    def run_port(sp):
        from oracle_bridge import Oracle
        from tis_gb300 import System
        s = System.load(files["pdb"], files["bonds"], files["stacks"], files["maxikey"], T=T_298, box=BOX, rc=RC,
                        center=500, rng=1, **sp)
        o = Oracle(s.to_dict(), seed=sp["seed"])
        o.populate_lists()
        t0 = time.perf_counter()
        o.step(steps)
        return time.perf_counter() - t0

    fn = run_ref if kind == "reference" else run_port
    with ThreadPoolExecutor(max_workers=workers) as ex:
        secs = list(ex.map(fn, sample))
    value = len(sample) * steps / max(secs)
    build = ("the reference engine (src/16SCD_Mg_Cl_K_COPY_fast.cpp with the four-item hook patch table), g++ "
             + " ".join(build_ref.BENCH_FLAGS) + ", single-rank MPI stub, glibc rand()") if exe else \
        "the C oracle port (oracle/tis_oracle.c), one thread per replica"
    return {"value": value, "unit": UNIT, "cores": len(sample), "kind": kind, "build": build,
            "sample": f"{len(sample)} of the {len(specs)} replicas ({steps} steps each, one per host core, "
                      f"concurrently; setup excluded)"}


N_BEADS = 3 * N_NT - 1  # the chain starts with a nucleotide: 1037 beads for 346 nt


def workload_config(specs):
    """The workload both arms run, with the sizes and conditions it is quoted on
    (identical dictionaries, so the two arms' lines name the same configuration)."""
    parts = [N_BEADS + sp["n_mg"] + sp["n_cl"] + sp["n_k"] for sp in specs]
    return {"workload": "64 replicas x 346-nt TIS chain (1037 beads) + Mg 0-20 mM sweep, 76 mM KCl, "
                        "350 A box, T 298 K, rc 30 A",
            "replicas_per_gpu": len(specs), "particles_per_gpu": int(sum(parts)),
            "particles_per_replica": [int(min(parts)), int(max(parts))],
            "box_A": BOX, "T_K": 298.0, "T_kcal_per_mol": T_298, "h": 0.05, "coulomb_cutoff_A": RC,
            "sr_list_A": 15.0, "lr_list_A": RC + 3.0, "lr_every_steps": 10, "mg_mM": [0.0, 20.0], "kcl_mM": 76.0,
            "seeds": [specs[0]["seed"], specs[-1]["seed"]],
            "l2": "GPU arm: flushed (256 MB write) before every timed graph replay"}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    with tempfile.TemporaryDirectory() as tmp:
        files = make_inputs(tmp)
        specs = replica_specs()
        workers = min(len(specs), os.cpu_count() or 1)
        cpu = cpu_sample(files, specs, max(200, args.steps), workers)
    line = {"impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * N_REPLICAS / cpu["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": workload_config(specs),
            "cpu_baseline": dict(cpu),
            "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def timed_steps(eng, K, W, flush, stream, world, clk_device):
    """EQUIL_STEPS untimed steps, W warm-up steps, every graph the timed region
    replays captured, then exactly K
    steps timed with CUDA events on the handle's stream: the step graph (graph_steps
    long) replayed K // graph_steps times and a graph of the remaining steps once,
    L2 flushed before each replay.  Returns (ms, launches, chunks, clock summary)."""
    import torch
    gs = eng.params.graph_steps
    chunks = [gs] * (K // gs) + ([K % gs] if K % gs else [])
    eng.step(EQUIL_STEPS)
    eng.step(W)
    for c in sorted(set(chunks), reverse=True):  # captures (the last one stays as the tail graph)
        eng.step(c)
    eng.sync()
    ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in chunks]
    if world > 1:
        torch.distributed.barrier()
    torch.cuda.synchronize()
    launches0 = eng.launches()
    host_s = 0.0
    with ClockSampler(clk_device) as clk:
        for i, c in enumerate(chunks):
            with torch.cuda.stream(stream):
                flush.zero_()  # L2 flush between timed replays (256 MB > 129 MB L2)
                ev[i][0].record(stream)
            t0 = time.perf_counter()
            eng.step(c)
            host_s += time.perf_counter() - t0
            with torch.cuda.stream(stream):
                ev[i][1].record(stream)
        eng.sync()
        torch.cuda.synchronize()
    ms = sum(a.elapsed_time(b) for a, b in ev)
    return ms, eng.launches() - launches0, chunks, clk.summary(), 1000.0 * host_s


def e2e_measure(eng, K, n_rep, reps=3):
    """End to end through the C ABI with host buffers, over the same K steps as the
    timed region, `reps` times: every replica's state uploaded from pinned host
    memory (tis_set_states), the lists rebuilt, K graph-replayed steps, a frame
    (positions and the five energies of every replica) read back into pinned host
    memory; host wall clock between device synchronisations."""
    import torch
    state = eng.get_states()
    pinned = {k: torch.from_numpy(v).pin_memory().numpy() for k, v in state.items()}
    frame = {k: torch.zeros(v.size, dtype=torch.float64).pin_memory().numpy() for k, v in state.items()
             if k in ("x", "y", "z")}
    energies = torch.zeros((n_rep, 5), dtype=torch.float64).pin_memory().numpy()
    h2d = sum(v.nbytes for v in pinned.values())
    d2h = sum(v.nbytes for v in frame.values()) + energies.nbytes

    def one():
        eng.set_states(pinned)
        eng.populate_lists()
        eng.step(K)
        eng.get_states(("x", "y", "z"), out=frame)
        eng.all_energies(out=energies)

    one()  # the same calls once untimed (graphs of these lengths captured)
    eng.sync()
    t0 = time.perf_counter()
    for _ in range(reps):
        one()
    eng.sync()
    dt = time.perf_counter() - t0
    return {"value": n_rep * K * reps / dt, "unit": UNIT, "h2d_bytes_per_step": h2d // K,
            "d2h_bytes_per_step": d2h // K, "steps_per_call": K, "repeats": reps,
            "calls": "tis_set_states (pinned) + tis_populate_lists + tis_step(K) + tis_get_states (x, y, z) + "
                     "tis_get_all_energies"}


def plain_steps_per_s(system, local, n_steps=500, precision=None):
    """One replica on its own handle, direct launches (no graph): the plain
    single-replica GPU path, timed with CUDA events on its stream."""
    import torch

    from tis_gb300 import PREC_FP64, Engine
    e = Engine([system], precision=PREC_FP64 if precision is None else precision, device=local, use_graph=0)
    e.populate_lists()
    e.step(50)
    e.sync()
    st = torch.cuda.ExternalStream(e.stream())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(st):
        a.record(st)
    e.step(n_steps)
    with torch.cuda.stream(st):
        b.record(st)
    e.sync()
    torch.cuda.synchronize()
    sps = n_steps / (a.elapsed_time(b) / 1000.0)
    e.close()
    return sps


def graph_steps_per_s(systems, local, n_steps, precision):
    """All `systems` on one handle, graph-replayed steps, CUDA events on its stream."""
    import torch

    from tis_gb300 import Engine
    e = Engine(systems, precision=precision, device=local, use_graph=1, graph_steps=n_steps)
    e.populate_lists()
    e.step(n_steps)
    e.sync()
    st = torch.cuda.ExternalStream(e.stream())
    a, b = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    with torch.cuda.stream(st):
        a.record(st)
    e.step(2 * n_steps)
    with torch.cuda.stream(st):
        b.record(st)
    e.sync()
    torch.cuda.synchronize()
    ms = a.elapsed_time(b)
    e.close()
    return len(systems) * 2 * n_steps / (ms / 1000.0), ms / (2 * n_steps)


def ref_one_core(files, kw, steps):
    """The reference engine (timing build) on one host core: steps/s, set-up excluded."""
    import build_ref
    exe = build_ref.build(bench=True)
    if not exe:
        return None
    args = [exe, "--pdb", files["pdb"], "--bonds", files["bonds"], "--stacks", files["stacks"],
            "--maxikey", files["maxikey"], "--steps", str(steps), "--time"]
    for k, v in kw.items():
        args += ["--" + k, str(v)]
    out = subprocess.run(args, check=True, capture_output=True, text=True).stdout
    return json.loads(out.strip().splitlines()[-1])["steps_per_s"]


def gpu_arm(args):
    import numpy as np
    import torch

    from tis_gb300 import PREC_FP64, PREC_MIXED, Engine, System, autotune, synth

    rank = int(os.environ.get("RANK", "0"))
    world = int(os.environ.get("WORLD_SIZE", "1"))
    local = int(os.environ.get("LOCAL_RANK", "0"))
    torch.cuda.set_device(local)
    if world > 1:
        import torch.distributed as dist
        dist.init_process_group("nccl")
    with tempfile.TemporaryDirectory() as tmp:
        files = make_inputs(tmp)
        specs = rank_replica_specs(rank)  # replicas only: every rank its own batch
        systems = load_systems(files, specs)
        # the launch configuration: measured by tis_autotune (replica groups, steps per
        # graph, threads per particle of the pair launches, step path) for calls of the
        # timed step count, each trial at least 1000 steps; or fixed by --groups
        tune = {"groups": args.groups, "graph_steps": args.graph_steps, "lanes_sr": args.lanes_sr,
                "lanes_lr": args.lanes_lr, "fused_ctas": args.fused_ctas}
        tune_s = None
        tune_note = "--groups"
        if args.groups == 0:
            t0 = time.perf_counter()
            try:
                tune, _ = autotune(systems, steps=max(1, args.steps), precision=PREC_MIXED, device=local)
                tune_note = f"tis_autotune (calls of {max(1, args.steps)} steps, at least 1000 steps per trial)"
            except Exception as exc:  # the library's defaults if tuning fails
                tune = {"groups": 0, "graph_steps": GRAPH_STEPS, "lanes_sr": 1, "lanes_lr": 4}
                tune_note = f"library defaults (tis_autotune failed: {exc})"
            tune_s = time.perf_counter() - t0
        eng = Engine(systems, precision=PREC_MIXED, device=local, use_graph=1, **tune)
        n_part = sum(eng.n)
        config = workload_config(specs)
        assert config["particles_per_gpu"] == n_part, (config["particles_per_gpu"], n_part)
        eng.populate_lists()
        stream = torch.cuda.ExternalStream(eng.stream())
        flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")
        K = max(1, args.steps)
        W = max(3, args.warmup)
        ms, launches, chunks, clocks, host_ms = timed_steps(eng, K, W, flush, stream, world, local)
        ms = max_over_ranks(ms, world, device=f"cuda:{local}")
        if world > 1:
            torch.distributed.barrier()
        ms_per_step = ms / K
        value = job_value(ms, world, N_REPLICAS, K)
        graph_steps = eng.params.graph_steps
        groups = eng.params.groups or (3 * N_REPLICAS + 15) // 16
        launch = {"path": "CUDA graph replay (one graph holds every replica group's branch)",
                  "graph_steps": graph_steps, "graph_launches": len(chunks), "chunks": chunks,
                  "equilibration_steps": EQUIL_STEPS,
                  "host_enqueue_ms": host_ms, "replica_groups": groups,
                  "lanes_sr": eng.params.lanes_sr or 1, "lanes_lr": eng.params.lanes_lr or 4,
                  "fused_ctas": eng.params.fused_ctas,
                  "config_source": tune_note, "autotune_s": tune_s}

        if not args.extras:
            if rank == 0:
                print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "steps": K,
                                  "ms_per_step": ms_per_step, "launch": launch,
                                  "note": "timed loop only (--no-extras)"}), flush=True)
            return

        e2e = e2e_measure(eng, K, N_REPLICAS) if rank == 0 else None

        # the plain single-replica FP64 GPU path on the central system (346-nt chain,
        # 129 Mg / 2219 Cl / 2307 K, 350 A box): the denominator of the batching target
        w1 = synth.WORKLOADS["central"]
        cfg1_sys = System.load(files["pdb"], files["bonds"], files["stacks"], files["maxikey"], T=T_298, box=BOX,
                               rc=RC, n_mg=w1["ions"][0], n_cl=w1["ions"][1], n_k=w1["ions"][2], seed=1,
                               center=500, rng=1)
        plain_sps = plain_steps_per_s(cfg1_sys, local)

        # in-step kernel times: every kernel timed inside the graph-replayed step with
        # all groups running concurrently (tis_profile_in_step), and each stage alone
        stages = eng.profile_stages(50)
        try:
            in_step = eng.profile_in_step(min(K, 100))
            in_step_src = "tis_profile_in_step"
        except Exception as exc:  # the stages run alone, per group, if the in-step capture fails
            in_step = {k: v / groups for k, v in stages.items()}
            in_step_src = f"tis_profile_stages (in-step capture failed: {exc})"
        peak, peak_kind = measured_peaks()
        cnt = [eng.counters(r) for r in range(N_REPLICAS)]
        reb_rep = sum(c[1] / max(1, c[0]) for c in cnt)  # replicas rebuilt per step
        nreb = reb_rep * n_part / N_REPLICAS
        sampled = [0, N_REPLICAS - 1]  # mean list lengths from two replicas (0 and 20 mM Mg)
        sr = sum(2 * len(eng.pairs(r, 0)) for r in sampled) / sum(eng.n[r] for r in sampled)
        lr = sum(2 * len(eng.pairs(r, 1)) for r in sampled) / sum(eng.n[r] for r in sampled)
        sd = systems[0].to_dict()
        nrna = int(np.asarray(sd["n_rna"]).ravel()[0]) * N_REPLICAS
        items = (len(sd["bt_kind"]) + len(sd["st3_E"]) + len(sd["st2_E"])) * N_REPLICAS
        nhb = len(sd["hb_E"]) * N_REPLICAS
        alg = stage_bytes(n_part, sr, lr, 0.1 + reb_rep / N_REPLICAS, nreb, nrna, items, nhb, N_REPLICAS)
        per_stage = {}
        for k in in_step:
            b = alg[k] / groups  # one launch = one replica group's kernel in one step
            per_stage[k] = {"in_step_us": 1000 * in_step[k], "alone_us_per_group": 1000 * stages[k] / groups,
                            "alg_bytes_per_launch": b,
                            "achieved_gbs": b / (in_step[k] * 1e-3) / 1e9 if in_step[k] > 0 else None}
        dom = max(stages, key=stages.get)  # the most execution time of its own (stages timed alone)
        ach = per_stage[dom]["achieved_gbs"]
        traffic = NCU_DRAM_BYTES_PER_REPLICA.get(dom)
        roofline = {"bound": "latency", "axis": "hbm", "kernel": dom, "achieved": ach, "peak": peak, "unit": "GB/s",
                    "frac": ach / peak, "peak_source": peak_kind,
                    "traffic": traffic * N_REPLICAS / groups if traffic is not None else None,
                    "alg_bytes_per_launch": per_stage[dom]["alg_bytes_per_launch"],
                    "launch_us_in_step": per_stage[dom]["in_step_us"],
                    "fp32_pipe_frac": NCU_FMA_PIPE.get(dom), "issue_active_frac": NCU_ISSUE_ACTIVE.get(dom),
                    "fp32_pair_sr": fp32_roofline(local, clocks, sr * n_part / groups, in_step.get("pair_sr", 0.0)),
                    "mean_neighbours": {"sr": sr, "lr": lr}, "stages": per_stage, "in_step_source": in_step_src,
                    "step": {"alg_bytes": sum(alg.values()),
                             "achieved_gbs": sum(alg.values()) / (ms_per_step * 1e-3) / 1e9,
                             "frac": sum(alg.values()) / (ms_per_step * 1e-3) / 1e9 / peak},
                    "note": "kernel with the most execution time of its own (each stage timed alone, "
                            "tis_profile_stages), timed inside the step (tis_profile_in_step: event pairs around "
                            "each kernel inside the concurrently replayed graphs of all groups); one launch = one "
                            "replica group (1/" + str(groups) + " of the batch) for one step; achieved = its "
                            "algorithmic bytes / its in-step duration; bound: the kernels are latency bound "
                            "(ncu: long-scoreboard stalls on dependent gathers, low DRAM and FP32-pipe use), "
                            "the axis is the measured HBM copy rate; fp32_pipe_frac and issue_active_frac "
                            "come from the committed ncu capture of that kernel; step: all stages' "
                            "algorithmic bytes per step over the timed step"}

        extras = {}
        if rank == 0:
            extras = more_configs(args, files, tmp, systems, local, cfg1_sys)

    if rank != 0:
        return
    cpu = cpu_sample(files_for_cpu(), replica_specs(), 2000, min(N_REPLICAS, os.cpu_count() or 1)) \
        if args.cpu_baseline else None
    line = {"metric": METRIC, "value": value, "unit": UNIT,
            "plain_fp64_single_replica_steps_per_s": plain_sps, "batched_vs_plain": value / world / plain_sps,
            "n_gpus": world, "steps": K, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+i64+f64", "data": "synthetic", "config": config, "launch": launch,
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu, "clocks": clocks,
            "precision": "mixed: FP32 pair/bonded math on exact fixed-point differences, int64 fixed-point force "
                         "sums, FP64 integration and energies"}
    line.update(extras)
    print(json.dumps(line), flush=True)


def n_particles(system):
    import numpy as np
    return int(np.asarray(system.to_dict()["n_particles"]).ravel()[0])


def more_configs(args, files, tmp, systems, local, cfg1_sys):
    """The benchmark description's other configurations, each on the GPU beside the
    reference engine where it names one; a configuration that fails is reported
    with its error instead of its numbers."""
    out = {}
    for name, fn in (("small_system_fp64", _cfg_small), ("central_single_replica", _cfg_central),
                     ("adjoint", _cfg_adjoint), ("large_system", _cfg_large)):
        if name == "large_system" and not args.large:
            continue
        try:
            out[name] = fn(args, files, tmp, local, cfg1_sys)
        except Exception as exc:
            out[name] = {"error": f"{type(exc).__name__}: {exc}"}
    return out


def _cfg_small(args, files, tmp, local, cfg1_sys):
    from tis_gb300 import System, synth
    # cfg 0: the 76-nt chain (227 beads) in a 200 A box with 10 Mg / 261 Cl / 317 K
    # (815 particles), FP64: the plain GPU path and the reference engine on one core
    w0 = synth.WORKLOADS["small"]
    f0 = synth.generate(tmp, "small", w0["n_nt"], seed=w0["seed"], n_hb_pairs=w0["n_hb_pairs"])
    s0 = System.load(f0["pdb"], f0["bonds"], f0["stacks"], f0["maxikey"], T=T_298, box=w0["box"], rc=RC,
                     n_mg=w0["ions"][0], n_cl=w0["ions"][1], n_k=w0["ions"][2], seed=1, center=100, rng=1)
    ref0 = ref_one_core(f0, dict(box=w0["box"], rc=RC, T=T_298, nMg=w0["ions"][0], nCl=w0["ions"][1],
                                 nK=w0["ions"][2], seed=1, center=100), 5000) if args.cpu_baseline else None
    return {"workload": "1 replica x 76-nt chain (227 beads) + 10 Mg / 261 Cl / 317 K, 200 A box, FP64",
            "particles": n_particles(s0), "plain_gpu_fp64_steps_per_s": plain_steps_per_s(s0, local, 1000),
            "reference_one_core_steps_per_s": ref0}


def _cfg_central(args, files, tmp, local, cfg1_sys):
    from tis_gb300 import PREC_MIXED
    # cfg 1: the central single replica (1037 beads + 129 Mg / 2219 Cl / 2307 K):
    # mixed precision from a graph, the plain FP64 path, the reference on one core
    mixed1, _ = graph_steps_per_s([cfg1_sys], local, 200, PREC_MIXED)
    ref1 = ref_one_core(files, dict(box=BOX, rc=RC, T=T_298, nMg=129, nCl=2219, nK=2307, seed=1, center=500),
                        1000) if args.cpu_baseline else None
    return {"workload": "1 replica x 346-nt chain (1037 beads) + 129 Mg / 2219 Cl / 2307 K, 350 A box",
            "particles": n_particles(cfg1_sys), "mixed_graph_steps_per_s": mixed1,
            "plain_gpu_fp64_steps_per_s": plain_steps_per_s(cfg1_sys, local, 500),
            "reference_one_core_steps_per_s": ref1}


def _cfg_adjoint(args, files, tmp, local, cfg1_sys):
    import numpy as np

    from tis_gb300 import PREC_MIXED, Engine, System
    # cfg 3: dU/dtheta of the 16 force-field parameters over 10^4 saved frames of the
    # central system (64 replicas with independent seeds, a frame every 10 steps),
    # uploaded 64 frames at a time from host memory; and the gradient through 200-step
    # fixed-noise trajectories with a checkpoint every 10 steps, 16 replicas
    base = cfg1_sys.to_dict()
    reps = [System.from_arrays(dict(base, seed=np.array([s], dtype=np.int64))) for s in range(1, 65)]
    fe = Engine(reps, precision=PREC_MIXED, device=local, use_graph=1, graph_steps=10)
    fe.populate_lists()
    n_frames = 10000
    template = fe.get_states()  # x_old and v of the uploads (dU/dtheta reads positions only)
    batches = []
    for _ in range((n_frames + 63) // 64):
        fe.step(10)
        batches.append(fe.get_states(("x", "y", "z")))
    fe.close()
    ge = Engine(reps, precision=PREC_MIXED, device=local, groups=1)
    ge.set_states(dict(template, **batches[0]))
    ge.populate_lists()
    ge.param_grad()
    ge.sync()
    t0 = time.perf_counter()
    for b in batches:
        ge.set_states(dict(template, **b))
        ge.populate_lists()
        ge.param_grad()
    ge.sync()
    t_pg = time.perf_counter() - t0
    ge.close()
    adj = Engine(reps[:16], precision=PREC_MIXED, device=local, groups=1)
    adj.populate_lists()
    adj.step(50)
    adj.sync()
    rng = np.random.default_rng(0)
    seed = {k: rng.standard_normal(sum(adj.n)) for k in ("x", "y", "z")}
    adj.traj_grad(20, 10, seed)
    t0 = time.perf_counter()
    adj.traj_grad(200, 10, seed)
    t_tg = time.perf_counter() - t0
    adj.close()
    return {
        "workload": "central system (346-nt chain + 129 Mg / 2219 Cl / 2307 K), 16 parameters",
        "param_grad_frames": 64 * len(batches), "param_grad_frames_per_s": 64 * len(batches) / t_pg,
        "param_grad_note": "frames uploaded from host memory 64 at a time, lists rebuilt, dU/dtheta; wall clock",
        "traj_replicas": 16, "traj_steps": 200, "checkpoint_every": 10, "traj_grad_s": t_tg,
        "traj_grad_replica_steps_per_s": 16 * 200 / t_tg,
        "precision": "mixed forward; adjoint in FP32 dual numbers with FP64 sums"}


def _cfg_large(args, files, tmp, local, cfg1_sys):
    # the large system, 16 replicas x 48,899 particles, graphs of GRAPH_STEPS steps
    import numpy as np

    from tis_gb300 import PREC_MIXED, System, synth
    w = synth.WORKLOADS["large"]
    lf = synth.generate(tmp, "large", w["n_nt"], seed=w["seed"], n_hb_pairs=w["n_hb_pairs"])
    m, cl, kk = w["ions"]
    lb = System.load(lf["pdb"], lf["bonds"], lf["stacks"], lf["maxikey"], T=T_298, box=w["box"], rc=RC,
                     n_mg=m, n_cl=cl, n_k=kk, seed=1, center=500, rng=1).to_dict()
    lreps = [System.from_arrays(dict(lb, seed=np.array([s], dtype=np.int64))) for s in range(1, 17)]
    sps, lms = graph_steps_per_s(lreps, local, GRAPH_STEPS, PREC_MIXED)
    return {"workload": "16 replicas x 1500-nt chain (4499 beads), 600 A box, 1300 Mg / 22100 Cl / 21000 K",
            "particles_per_replica": n_particles(lreps[0]), "ms_per_step": lms, "replica_steps_per_s": sps,
            "precision": "mixed"}


def profile_fused(args):
    """The fused step kernel's phase times on the 64-replica workload (one replica
    group), cluster sizes 1, 2 and 4: 20 steps to settle, then args.steps timed."""
    from tis_gb300 import PREC_MIXED, Engine
    with tempfile.TemporaryDirectory() as tmp:
        systems = load_systems(make_inputs(tmp), replica_specs())
        for ctas in (1, 2, 4):
            e = Engine(systems, precision=PREC_MIXED, groups=1, fused_ctas=ctas)
            e.populate_lists()
            e.profile_fused(20, ctas)
            ph = e.profile_fused(max(1, args.steps), ctas)
            print(json.dumps({"fused_ctas": ctas, "replicas": len(systems), "steps": args.steps, **ph}), flush=True)
            e.close()


def files_for_cpu():
    d = tempfile.mkdtemp()
    return make_inputs(d)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--gpus", type=int, default=1)
    ap.add_argument("--steps", type=int, default=2000)
    ap.add_argument("--warmup", type=int, default=5)
    ap.add_argument("--impl", default="gpu", choices=["gpu", "reference"])
    ap.add_argument("--groups", type=int, default=0,
                    help="fixed launch configuration: replica groups run concurrently (0: tis_autotune chooses "
                         "groups, steps per graph and pair-launch shapes)")
    ap.add_argument("--graph-steps", type=int, default=GRAPH_STEPS, help="steps per graph with --groups")
    ap.add_argument("--lanes-sr", type=int, default=1, help="SR pair threads per particle with --groups")
    ap.add_argument("--lanes-lr", type=int, default=4, help="LR pair threads per particle with --groups")
    ap.add_argument("--fused-ctas", type=int, default=0,
                    help="with --groups: CTAs per replica of the persistent fused step kernel (0: separate kernels)")
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-large", dest="large", action="store_false",
                    help="skip the large-system (48,899 particles x 16 replicas) throughput line")
    ap.add_argument("--profile-fused", action="store_true",
                    help="instead of the benchmark: the persistent fused step kernel's phase times "
                         "(tis_profile_fused) on the workload, one line per cluster size")
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="stop after the timed loop (no e2e, stage timing, plain path): for profiler runs")
    args = ap.parse_args()
    if args.profile_fused:
        profile_fused(args)
    elif args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
