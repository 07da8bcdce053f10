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

--impl reference times the reference's own CPU engine (oracle/_ref/tis_ref, built
from the reference sources; else the C oracle port) on the host cores, one
replica per core, on a bounded sample of the same workload.
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
NCU_DRAM_BYTES_PER_REPLICA = {"pair_sr": 3.04e6 / 8, "pair_lr": None, "bonded": 1.24e6 / 8, "hbond": 0.48e6 / 8,
                              "shift": 0.04e6 / 8, "integrate": 5.35e6 / 8, "cells": 0.03e6 / 8, "search": None}


def cpu_sample(files, specs, steps, workers):
    """Reference CPU engine on `workers` replicas in parallel, `steps` steps each."""
    import build_ref
    exe = build_ref.build()
    kind = "reference" if exe else "port"
    sample = specs[:: max(1, len(specs) // workers)][:workers]

    def run_ref(sp):
        args = [exe, "--pdb", files["pdb"], "--bonds", files["bonds"], "--stacks", files["stacks"],
                "--maxikey", files["maxikey"], "--box", str(BOX), "--rc", str(RC), "--T", str(T_298),
                "--nMg", str(sp["n_mg"]), "--nCl", str(sp["n_cl"]), "--nK", str(sp["n_k"]),
                "--seed", str(sp["seed"]), "--center", "500", "--rng", "philox", "--steps", str(steps), "--time"]
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
    return {"value": value, "unit": UNIT, "cores": len(sample), "kind": kind,
            "sample": f"{len(sample)} of the {len(specs)} replicas ({steps} steps each, one per host core, "
                      f"concurrently; setup excluded)"}


def reference_arm(args):
    rank = int(os.environ.get("RANK", "0"))
    if rank != 0:
        return
    with tempfile.TemporaryDirectory() as tmp:
        files = make_inputs(tmp)
        specs = replica_specs()
        workers = min(len(specs), os.cpu_count() or 1)
        cpu = cpu_sample(files, specs, max(200, args.steps), workers)
    cpu_line = dict(cpu)
    line = {"impl": "reference", "metric": METRIC, "value": cpu["value"], "unit": UNIT, "n_gpus": args.gpus,
            "steps": args.steps, "warmup": args.warmup, "ms_per_step": 1000.0 * N_REPLICAS / cpu["value"],
            "higher_is_better": True, "scaling": "weak", "vs_baseline": None, "dtype": "f64", "data": "synthetic",
            "config": {"workload": "64 replicas x 346-nt TIS chain + Mg 0-20 mM sweep, 76 mM KCl, 350 A box",
                       "replicas": N_REPLICAS},
            "cpu_baseline": cpu_line,
            "e2e": {"value": cpu["value"], "unit": UNIT, "h2d_bytes_per_step": 0, "d2h_bytes_per_step": 0}}
    print(json.dumps(line), flush=True)


def gpu_arm(args):
    import numpy as np
    import torch

    from tis_gb300 import PREC_FP64, PREC_MIXED, Engine, autotune

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
        # graph, threads per particle of the pair launches; 1000 steps per trial), or
        # fixed by --groups
        tune = {"groups": args.groups, "graph_steps": args.graph_steps, "lanes_sr": args.lanes_sr,
                "lanes_lr": args.lanes_lr}
        tune_s = None
        tune_note = "--groups"
        if args.groups == 0:
            t0 = time.perf_counter()
            try:
                tune, _ = autotune(systems, steps=1000, precision=PREC_MIXED, device=local)
                tune_note = "tis_autotune (1000 steps per trial)"
            except Exception as exc:  # the library's defaults if tuning fails
                tune = {"groups": 0, "graph_steps": GRAPH_STEPS, "lanes_sr": 1, "lanes_lr": 4}
                tune_note = f"library defaults (tis_autotune failed: {exc})"
            tune_s = time.perf_counter() - t0
        eng = Engine(systems, precision=PREC_MIXED, device=local, use_graph=1, **tune)
        graph_steps = eng.params.graph_steps
        eng.populate_lists()
        stream = torch.cuda.ExternalStream(eng.stream())
        flush = torch.empty(256 * 1024 * 1024, dtype=torch.uint8, device=f"cuda:{local}")
        K = max(1, args.steps)
        W = max(3, args.warmup)
        eng.step(W)                # W warm-up steps (direct launches) ...
        eng.step(graph_steps)      # ... and one graph replay, so capture happens before timing
        eng.sync()
        chunks = [graph_steps] * (K // graph_steps) + ([K % graph_steps] if K % graph_steps else [])
        iters = len(chunks)
        ev = [(torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)) for _ in range(iters)]
        if world > 1:
            torch.distributed.barrier()
        torch.cuda.synchronize()
        launches0 = eng.launches()
        with ClockSampler(local) as clk:
            for i in range(iters):
                with torch.cuda.stream(stream):
                    flush.zero_()  # L2 flush between timed iterations (256 MB > 129 MB L2)
                    ev[i][0].record(stream)
                eng.step(chunks[i])
                with torch.cuda.stream(stream):
                    ev[i][1].record(stream)
            eng.sync()
            torch.cuda.synchronize()
        ms = sum(a.elapsed_time(b) for a, b in ev)
        launches = eng.launches() - launches0
        ms = max_over_ranks(ms, world, device=f"cuda:{local}")
        if world > 1:
            torch.distributed.barrier()
        ms_per_step = ms / K
        value = job_value(ms, world, N_REPLICAS, K)

        if not args.extras:
            if rank == 0:
                print(json.dumps({"metric": METRIC, "value": value, "unit": UNIT, "steps": K,
                                  "ms_per_step": ms_per_step, "note": "timed loop only (--no-extras)"}), flush=True)
            return

        # end to end through the C ABI with host buffers: every 100 steps every
        # replica's state is uploaded from pinned host memory (one call), the lists
        # are rebuilt, 100 steps run, and a frame (positions + the five energies of
        # every replica) is read back into pinned host memory
        e2e = None
        if rank == 0:
            E2E_STEPS = max(100, graph_steps)  # whole graphs between frames
            n_it = max(1, min(10, K // E2E_STEPS))
            state = eng.get_states()
            pinned = {k: torch.from_numpy(v).pin_memory().numpy() for k, v in state.items()}
            frame = {k: torch.zeros(v.size, dtype=torch.float64).pin_memory().numpy() for k, v in state.items()
                     if k in ("x", "y", "z")}
            energies = torch.zeros((N_REPLICAS, 5), dtype=torch.float64).pin_memory().numpy()
            h2d = sum(v.nbytes for v in pinned.values())
            d2h = sum(v.nbytes for v in frame.values()) + energies.nbytes
            t0 = time.perf_counter()
            for _ in range(n_it):
                eng.set_states(pinned)
                eng.populate_lists()
                eng.step(E2E_STEPS)
                eng.get_states(("x", "y", "z"), out=frame)
                eng.all_energies(out=energies)
            eng.sync()
            dt = time.perf_counter() - t0
            e2e = {"value": N_REPLICAS * E2E_STEPS * n_it / dt, "unit": UNIT,
                   "h2d_bytes_per_step": h2d // E2E_STEPS, "d2h_bytes_per_step": d2h // E2E_STEPS,
                   "frame_every_steps": E2E_STEPS}

        # per-stage device time: each stage's kernels alone, CUDA events between them on
        # the group streams, ms per step summed over the replica groups
        stages = eng.profile_stages(50)
        peak, peak_kind = measured_peaks()
        n_part = sum(eng.n)
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
        for k, ms_k in stages.items():
            gbs = alg[k] / (ms_k * 1e-3) / 1e9 if ms_k > 0 else None
            per_stage[k] = {"ms": ms_k, "alg_bytes": alg[k], "achieved_gbs": gbs,
                            "frac": gbs / peak if gbs is not None else None}
        dom = max(stages, key=stages.get)
        traffic = NCU_DRAM_BYTES_PER_REPLICA.get(dom)
        roofline = {"bound": "hbm", "kernel": dom, "achieved": per_stage[dom]["achieved_gbs"], "peak": peak,
                    "unit": "GB/s", "frac": per_stage[dom]["frac"],
                    "traffic": traffic * N_REPLICAS if traffic is not None else None,
                    "alg_bytes_per_launch": alg[dom], "peak_source": peak_kind,
                    "mean_neighbours": {"sr": sr, "lr": lr}, "stages": per_stage,
                    "step": {"alg_bytes": sum(alg.values()),
                             "achieved_gbs": sum(alg.values()) / (ms_per_step * 1e-3) / 1e9,
                             "frac": sum(alg.values()) / (ms_per_step * 1e-3) / 1e9 / peak,
                             "note": "every stage's algorithmic bytes of one step of the batch over the "
                                     "graph-replayed step time"},
                    "note": "stage = its kernels over all replica groups run alone; launch = one step of "
                            "the batch; the integrator is FP64-pipe bound, the H-bond kernel latency bound "
                            "(serial Monte Carlo per replica)"}

        # the plain single-replica FP64 GPU path (the denominator of the batching target)
        plain = Engine([systems[len(systems) // 2]], precision=PREC_FP64, device=local, use_graph=0)
        plain.populate_lists()
        plain.step(50)
        plain.sync()
        t0e, t1e = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
        pstream = torch.cuda.ExternalStream(plain.stream())
        NP = 500
        with torch.cuda.stream(pstream):
            t0e.record(pstream)
        plain.step(NP)
        with torch.cuda.stream(pstream):
            t1e.record(pstream)
        plain.sync()
        torch.cuda.synchronize()
        plain_sps = NP / (t0e.elapsed_time(t1e) / 1000.0)
        plain.close()

        # the differentiation workload: 16 replicas of the chain, dU/dtheta of 15
        # parameters at their current frames, and the gradient through a 200-step
        # fixed-noise trajectory with a checkpoint every 10 steps (forward, recomputation
        # and reverse pass in one call); host wall clock around synchronous calls
        adjoint = None
        if rank == 0:
            adj = Engine(systems[:16], precision=PREC_MIXED, device=local, groups=1)  # the adjoint runs group by group
            adj.populate_lists()
            adj.step(50)
            adj.sync()
            adj.param_grad()
            t0 = time.perf_counter()
            for _ in range(5):
                adj.param_grad()
            t_pg = (time.perf_counter() - t0) / 5
            rng = np.random.default_rng(0)
            seed = {k: rng.standard_normal(sum(adj.n)) for k in ("x", "y", "z")}
            adj.traj_grad(20, 10, seed)
            t0 = time.perf_counter()
            adj.traj_grad(200, 10, seed)
            t_tg = time.perf_counter() - t0
            adjoint = {"replicas": 16, "param_grad_frames_per_s": 16 / t_pg,
                       "traj_steps": 200, "checkpoint_every": 10, "traj_grad_s": t_tg,
                       "traj_grad_replica_steps_per_s": 16 * 200 / t_tg,
                       "precision": "mixed forward; adjoint in FP32 dual numbers with FP64 sums"}
            adj.close()

        # the large system: a 1500-nt chain in a 600 A box with 1300 Mg, 22100 Cl,
        # 21000 K (48,899 particles per replica), 16 replicas with independent seeds
        # (one set-up, the seed varied), mixed precision, graphs of GRAPH_STEPS steps
        large = None
        if rank == 0 and args.large:
            from tis_gb300 import System, synth
            w = synth.WORKLOADS["large"]
            lf = synth.generate(tmp, "large", w["n_nt"], seed=w["seed"], n_hb_pairs=w["n_hb_pairs"])
            m, cl, kk = w["ions"]
            base = System.load(lf["pdb"], lf["bonds"], lf["stacks"], lf["maxikey"], T=T_298, box=w["box"], rc=RC,
                               n_mg=m, n_cl=cl, n_k=kk, seed=1, center=500, rng=1).to_dict()
            reps = [System.from_arrays(dict(base, seed=np.array([s], dtype=np.int64))) for s in range(1, 17)]
            le = Engine(reps, precision=PREC_MIXED, device=local, use_graph=1, graph_steps=GRAPH_STEPS)
            le.populate_lists()
            le.step(GRAPH_STEPS)
            le.sync()
            ls = torch.cuda.ExternalStream(le.stream())
            a0, a1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
            LN = 3 * GRAPH_STEPS
            with torch.cuda.stream(ls):
                a0.record(ls)
            le.step(LN)
            with torch.cuda.stream(ls):
                a1.record(ls)
            le.sync()
            torch.cuda.synchronize()
            lms = a0.elapsed_time(a1)
            large = {"workload": "16 replicas x 1500-nt chain (4499 beads), 600 A box, 1300 Mg / 22100 Cl / 21000 K",
                     "particles_per_replica": le.n[0], "steps": LN, "ms_per_step": lms / LN,
                     "replica_steps_per_s": 16 * LN / (lms / 1000.0), "precision": "mixed"}
            le.close()

    if rank != 0:
        return
    cpu = cpu_sample(files_for_cpu(), replica_specs(), 2000, min(N_REPLICAS, os.cpu_count() or 1)) \
        if args.cpu_baseline else None
    line = {"metric": METRIC, "value": value, "unit": UNIT, "n_gpus": world, "steps": K, "warmup": args.warmup,
            "ms_per_step": ms_per_step, "higher_is_better": True, "scaling": "weak", "vs_baseline": None,
            "dtype": "f32+i64+f64", "data": "synthetic",
            "config": {"workload": "64 replicas x 346-nt TIS chain (1037 beads) + Mg 0-20 mM sweep, 76 mM KCl, "
                                   "350 A box, T 298 K, rc 30 A",
                       "replicas_per_gpu": N_REPLICAS, "particles_per_gpu": n_part, "precision": "mixed",
                       "graph_steps": graph_steps, "replica_groups": eng.params.groups or (3 * N_REPLICAS + 15) // 16,
                       "lanes_sr": eng.params.lanes_sr or 1, "lanes_lr": eng.params.lanes_lr or 4,
                       "launch_config": tune_note,
                       "autotune_s": tune_s,
                       "l2": "flushed (256 MB write) between timed iterations of "
                                                         f"{graph_steps} steps", "parallelism": f"replicas x{world}"},
            "plain_fp64_single_replica_steps_per_s": plain_sps,
            "batched_vs_plain": value / world / plain_sps,
            "stage_ms_per_step": stages,
            "e2e": e2e, "gpu_launches": launches, "roofline": roofline, "cpu_baseline": cpu, "adjoint": adjoint,
            "large_system": large,
            "clocks": clk.summary()}
    print(json.dumps(line), flush=True)


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
    ap.add_argument("--no-cpu-baseline", dest="cpu_baseline", action="store_false")
    ap.add_argument("--no-large", dest="large", action="store_false",
                    help="skip the large-system (48,899 particles x 16 replicas) throughput line")
    ap.add_argument("--no-extras", dest="extras", action="store_false",
                    help="stop after the timed loop (no e2e, stage timing, plain path): for profiler runs")
    args = ap.parse_args()
    if args.impl == "reference":
        reference_arm(args)
    else:
        gpu_arm(args)


if __name__ == "__main__":
    main()
