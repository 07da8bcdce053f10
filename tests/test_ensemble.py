"""Stochastic runs reproduce the FP64 oracle's ensemble means within statistical
error.

Three independent ensembles of the 76-nt system (64 replicas each, distinct seeds,
so distinct ion placements, noise and Monte Carlo draws): the C oracle's (the
reference's algorithm and arithmetic, pinned to the reference engine), and the GPU
engine's in mixed precision and on its FP64 path.  Every replica runs 1000 steps
of relaxation, then 8000 steps sampled every 100.  Observables: the Energies-file
values (E2_HB, E3_HB, E2_STACK, E3_STACK, Rg; E:6308-6312) and the ions within 5 A
of a phosphate, Mg and K, counted per phosphate and summed (the counting radius of
analysis/salt_nt/dcd_traj_SaltCount_Kinetics_PBC.py:40-46).  Each replica's time
average is one sample; each GPU ensemble's mean must lie within 4 standard errors
of the difference from the oracle ensemble's mean."""
import os
from concurrent.futures import ThreadPoolExecutor

import numpy as np
import pytest

from oracle_bridge import Oracle
from systems import golden_inputs, load
from tis_gb300 import PREC_FP64, PREC_MIXED, Engine

pytestmark = pytest.mark.gpu

N_REP = 64
RELAX, SAMPLES, EVERY = 1000, 80, 100
NAMES = ["E2_HB", "E3_HB", "E2_STACK", "E3_STACK", "Rg", "Mg_5A", "K_5A"]
KIND_P, KIND_MG, KIND_K = 0, 3, 5


def _gpu_ensemble(prec, seeds):
    systems = [load(golden_inputs(), "small", seed=s) for s in seeds]
    e = Engine(systems, precision=prec)
    e.populate_lists()
    e.step(RELAX)
    samples = []
    for _ in range(SAMPLES):
        e.step(EVERY)
        en = e.all_energies()
        ions = np.array([[e.ion_counts(r, kind, 5.0)[0].sum() for kind in (KIND_MG, KIND_K)] for r in range(N_REP)])
        samples.append(np.concatenate([en, ions], axis=1))
    e.close()
    return np.mean(samples, axis=0)  # replicas x observables: time averages


def _bound_ions(st, kind, box, cut=5.0):
    """Ions of `kind` within `cut` of each phosphate, summed over the phosphates
    (minimum image)."""
    X = np.stack([st["x"], st["y"], st["z"]], 1)
    P = X[kind == KIND_P]
    out = []
    for k in (KIND_MG, KIND_K):
        Ion = X[kind == k]
        dv = P[:, None, :] - Ion[None, :, :]
        dv -= box * np.round(dv / box)
        out.append(int(((dv * dv).sum(-1) <= cut * cut).sum()))
    return out


def _oracle_replica(seed):
    s = load(golden_inputs(), "small", seed=seed)
    sd = s.to_dict()
    kind = np.asarray(sd["kind"])
    box = np.asarray(sd["box"], dtype=np.float64)
    o = Oracle(sd, seed=seed)
    o.populate_lists()
    o.step(RELAX)
    rows = []
    for _ in range(SAMPLES):
        o.step(EVERY)
        rows.append(np.concatenate([o.last_energies(), _bound_ions(o.get_state(), kind, box)]))
    return np.mean(rows, axis=0)


def _oracle_ensemble(seeds):
    # the oracle's calls release the GIL (ctypes), so threads run replicas in parallel
    with ThreadPoolExecutor(max_workers=min(len(seeds), os.cpu_count() or 1)) as ex:
        return np.array(list(ex.map(_oracle_replica, seeds)))


@pytest.fixture(scope="module")
def oracle_means():
    return _oracle_ensemble(list(range(300, 300 + N_REP)))


def _compare(a, b, label):
    rows = []
    for k, name in enumerate(NAMES):
        ma, mb = a[:, k].mean(), b[:, k].mean()
        se = np.sqrt(a[:, k].var(ddof=1) / len(a) + b[:, k].var(ddof=1) / len(b))
        z = (ma - mb) / se if se > 0 else 0.0
        rows.append(f"{name:9s} {label} {ma:+.5e} oracle {mb:+.5e} diff/se {z:+.2f}")
    print("\n".join(rows))
    for k, row in enumerate(rows):
        ma, mb = a[:, k].mean(), b[:, k].mean()
        se = np.sqrt(a[:, k].var(ddof=1) / len(a) + b[:, k].var(ddof=1) / len(b))
        assert abs(ma - mb) <= 4 * se + 1e-12 * max(abs(ma), abs(mb)), row


def test_mixed_ensemble_matches_oracle_ensemble(oracle_means):
    _compare(_gpu_ensemble(PREC_MIXED, range(100, 100 + N_REP)), oracle_means, "mixed")


def test_fp64_ensemble_matches_oracle_ensemble(oracle_means):
    _compare(_gpu_ensemble(PREC_FP64, range(200, 200 + N_REP)), oracle_means, "fp64 ")
