"""Stochastic runs reproduce ensemble means within statistical error.

Two independent ensembles of the 76-nt system (64 replicas each, distinct seeds,
so distinct ion placements and noise): one in mixed precision, one on the FP64
path (which follows the oracle's trajectories step for step, see
test_gpu_parity.py).  Observables, sampled every 100 steps over 8000 steps after
1000 steps of relaxation: the Energies-file values (E2_HB, E3_HB, E2_STACK,
E3_STACK, Rg) and the ions within 5 A of a phosphate (Mg and K, counted per
phosphate and summed; the reference's analysis/salt_nt counting radius).  Each
replica's time average is one sample; the ensembles' means must agree within
4 standard errors of their difference."""
import numpy as np
import pytest

from systems import golden_inputs, load
from tis_gb300 import PREC_FP64, PREC_MIXED, Engine

pytestmark = pytest.mark.gpu

N_REP = 64
NAMES = ["E2_HB", "E3_HB", "E2_STACK", "E3_STACK", "Rg", "Mg_5A", "K_5A"]


def _ensemble(prec, seeds):
    systems = [load(golden_inputs(), "small", seed=s) for s in seeds]
    e = Engine(systems, precision=prec)
    e.populate_lists()
    e.step(1000)
    samples = []
    for _ in range(80):
        e.step(100)
        en = e.all_energies()
        ions = np.array([[e.ion_counts(r, kind, 5.0)[0].sum() for kind in (3, 5)] for r in range(N_REP)])
        samples.append(np.concatenate([en, ions], axis=1))
    e.close()
    return np.mean(samples, axis=0)  # replicas x observables: time averages


def test_mixed_and_fp64_ensemble_means_agree():
    a = _ensemble(PREC_MIXED, range(100, 100 + N_REP))
    b = _ensemble(PREC_FP64, range(200, 200 + N_REP))
    rows = []
    for k, name in enumerate(NAMES):
        ma, mb = a[:, k].mean(), b[:, k].mean()
        se = np.sqrt(a[:, k].var(ddof=1) / N_REP + b[:, k].var(ddof=1) / N_REP)
        rows.append(f"{name:9s} mixed {ma:+.5e} fp64 {mb:+.5e} diff/se {(ma - mb) / se if se > 0 else 0:+.2f}")
        assert abs(ma - mb) <= 4 * se + 1e-12 * max(abs(ma), abs(mb)), rows[-1]
    print("\n".join(rows))
