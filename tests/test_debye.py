"""The screened (Debye-Hueckel) Coulomb term q_i q_j lB exp(-r / lambda_D) / r.

The reference has plain truncated Coulomb (E:825-855), which is lambda_D = 0 or
infinity here, the default; a finite Debye length is an addition.  Checked:
  * unscreened (no "debye" scalar, 0 or infinity) runs are bit-identical;
  * with lambda_D = 10 A the SR and LR Coulomb forces and energies match the FP64
    oracle patched with the same factor, per term: relative 1e-5 (mixed),
    1e-10 (FP64), on a thermal frame of the 76-nt and the central systems;
  * dU/dtheta of all 16 parameters, the Debye length among them, against central
    differences (h = 1e-4 relative) of the engine's and the oracle's FP64 energy;
  * dL/dlambda_D and dL/dlB through 40 fixed-noise FP64 steps against central
    differences of the engine's trajectories (h = 1e-3 relative).
"""
import numpy as np
import pytest

from oracle_bridge import Oracle
from systems import golden_inputs, load, rel_err
from tis_autograd import params_of, run_final_state, screened, with_params
from tis_gb300 import (N_PARAMS, PARAM_NAMES, PREC_FP64, PREC_MIXED, TERM_BONDED, TERM_HB, TERM_LR, TERM_SR,
                       TERM_STACK, Engine)

pytestmark = pytest.mark.gpu

DEBYE = 10.0
ALL = TERM_SR | TERM_LR | TERM_BONDED | TERM_STACK | TERM_HB
U_TERMS = ["E_lj", "E_coul_sr", "E_coul_lr", "E_bond", "E_angle", "E_excl", "E2_STACK", "E3_STACK", "E2_HB", "E3_HB"]


@pytest.fixture(scope="module")
def systems(synth_dir):
    return {"small": load(golden_inputs(), "small"), "central": load(synth_dir["central"], "central")}


def _thermal(system, steps=300):
    e = Engine([system], precision=PREC_FP64)
    e.populate_lists()
    e.step(steps)
    e.sync()
    st = e.get_states()
    e.close()
    return st


@pytest.fixture(scope="module")
def thermal(systems):
    return {k: _thermal(s) for k, s in systems.items()}


def test_unscreened_settings_are_bit_identical(systems):
    s = systems["small"]
    runs = []
    for sysobj in (s, screened(s, 0.0), screened(s, np.inf)):
        e = Engine([sysobj])
        e.populate_lists()
        e.step(200)
        e.sync()
        runs.append(e.get_state(0))
        e.close()
    for r in runs[1:]:
        for k in r:
            assert np.array_equal(r[k], runs[0][k]), k


@pytest.mark.parametrize("prec_name,prec,tol", [("mixed", PREC_MIXED, 1e-5), ("fp64", PREC_FP64, 1e-10)])
@pytest.mark.parametrize("case", ["small", "central"])
def test_screened_coulomb_terms_match_oracle(systems, thermal, case, prec_name, prec, tol):
    s = screened(systems[case], DEBYE)
    st = thermal[case]
    o = Oracle(s.to_dict(), seed=3)
    o.set_state(st)
    o.populate_lists()
    ref = o.terms()
    plain = Oracle(systems[case].to_dict(), seed=3)
    plain.set_state(st)
    plain.populate_lists()
    unscr = plain.terms()
    # the screening changes the LR term by far more than the tolerance
    assert rel_err(ref["F_lr"], unscr["F_lr"]) > 0.5
    report = []
    for name, mask, ek in (("F_sr", TERM_SR, ["E_lj", "E_coul_sr"]), ("F_lr", TERM_LR, ["E_coul_lr"])):
        e = Engine([s], precision=prec)
        e.set_states(st)
        e.populate_lists()
        f, en = e.forces(0, mask)
        e.close()
        want = ref[name]
        rel = rel_err(f, want)
        mx = np.abs(f - want).max() / np.abs(want).max()
        report.append(f"{name} rel {rel:.2e} max {mx:.2e}")
        assert rel <= tol and mx <= tol, (name, rel, mx)
        for k in ek:
            assert en[k] == pytest.approx(ref[k], rel=tol, abs=tol * max(1.0, abs(ref[k]))), (name, k)
    print(f"{case} debye {DEBYE} A {prec_name}: " + "; ".join(report))


def _potential(system, theta, state):
    e = Engine([with_params(system, theta)], precision=PREC_FP64)
    e.set_states(state)
    e.populate_lists()
    _, en = e.forces(0, ALL)
    e.close()
    return sum(en[k] for k in U_TERMS), sum(abs(en[k]) for k in U_TERMS)


def _oracle_potential(system, theta, state):
    o = Oracle(with_params(system, theta).to_dict(), seed=int(system["seed"][0]))
    o.set_state(state)
    o.populate_lists()
    t = o.terms()
    return sum(t[k] for k in U_TERMS)


def test_screened_param_grad_matches_finite_differences(systems, thermal):
    s = screened(systems["small"], DEBYE)
    st = thermal["small"]
    th0 = params_of(s)
    assert th0[15] == DEBYE
    e = Engine([s], precision=PREC_FP64)
    e.set_states(st)
    g = e.param_grad()[0]
    e.close()
    u0, uabs = _potential(s, th0, st)
    u1, _ = _potential(s, th0, st)
    noise = max(abs(u1 - u0), 1e-14 * uabs)
    rows = []
    for j in range(N_PARAMS):
        hj = 1e-4 * abs(th0[j])
        tp, tm = th0.copy(), th0.copy()
        tp[j] += hj
        tm[j] -= hj
        fd = (_potential(s, tp, st)[0] - _potential(s, tm, st)[0]) / (2 * hj)
        ofd = (_oracle_potential(s, tp, st) - _oracle_potential(s, tm, st)) / (2 * hj)
        rows.append(f"{PARAM_NAMES[j]:7s} adj {g[j]:+.9e} fd {fd:+.9e} oracle fd {ofd:+.9e}")
        assert abs(g[j] - fd) <= 1e-4 * abs(fd) + 10 * noise / hj, rows[-1]
        assert abs(g[j] - ofd) <= 1e-4 * abs(ofd) + 1e-14 * abs(u0) / hj, rows[-1]
    print("\n".join(rows))
    assert g[15] != 0.0


def _loss(state, seed):
    return sum(float(np.dot(state[k], w)) for k, w in seed.items())


def test_screened_traj_grad_matches_finite_differences(systems, thermal):
    s = screened(systems["small"], DEBYE)
    st = thermal["small"]
    th0 = params_of(s)
    rng = np.random.default_rng(5)
    seed = {k: rng.standard_normal(st["x"].size) for k in ("x", "y", "z", "vx", "vy", "vz")}
    e = Engine([s], precision=PREC_FP64)
    e.set_states(st)
    dth = e.traj_grad(40, 10, seed)[0]
    e.close()
    L = [_loss(run_final_state(s, th0, st, 40, precision=PREC_FP64), seed) for _ in range(3)]
    noise = max(max(L) - min(L), 1e-14 * abs(L[0]))
    rows = []
    for j in (14, 15):  # lB and the Debye length
        hj = 1e-3 * abs(th0[j])
        tp, tm = th0.copy(), th0.copy()
        tp[j] += hj
        tm[j] -= hj
        fd = (_loss(run_final_state(s, tp, st, 40, precision=PREC_FP64), seed) -
              _loss(run_final_state(s, tm, st, 40, precision=PREC_FP64), seed)) / (2 * hj)
        rows.append(f"{PARAM_NAMES[j]:7s} adj {dth[j]:+.9e} fd {fd:+.9e}")
        assert abs(dth[j] - fd) <= 1e-4 * abs(fd) + noise / hj, rows[-1]
    print("\n".join(rows))
