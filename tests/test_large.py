"""The large system of the benchmark description: a seeded 1500-nt chain (4499
beads, 400 H-bond pairs) in a 600 A box with 1300 Mg, 22100 Cl and 21000 K
(48,899 particles), 16 replicas batched with independent seeds.

  * cells, SR/LR pair sets and H-bond status: bit-exact against the oracle;
  * per-term forces and energies on the set-up frame: 1e-5 (mixed), 1e-10 (FP64);
  * forces and energies against the FP64 oracle on 100 frames sampled from a
    batched mixed-precision run of the 16 replicas: the step's total force (the
    hot path, which leaves a bonded pair's LJ out of the pair sum instead of
    adding and subtracting it) against the oracle's total formed the same way,
    and the LR, stacking and H-bond terms with their energies; the largest
    relative error over the frames is reported and held to 1e-5.  (The per-term
    SR and bonded split carries the LJ of a folded 1-3 pair twice, 1e17 kcal/mol/A
    and more, beyond the fixed-point range: on such frames the mixed per-term call
    reports TIS_ERR_NONFINITE, so those two terms are checked through the total.)"""
import numpy as np
import pytest

from oracle_bridge import Oracle
from systems import pair_set, rel_err
from tis_gb300 import (PREC_FP64, PREC_MIXED, STATE_NAMES, TERM_BONDED, TERM_HB, TERM_LR, TERM_SR, TERM_STACK,
                       Engine, System, synth)

pytestmark = pytest.mark.gpu

TERMS = [("F_hb", TERM_HB), ("F_sr", TERM_SR), ("F_lr", TERM_LR), ("F_bonded", TERM_BONDED), ("F_stack", TERM_STACK)]
E_TERM = {"F_sr": ["E_lj", "E_coul_sr"], "F_lr": ["E_coul_lr"], "F_bonded": ["E_bond", "E_angle", "E_excl"],
          "F_stack": ["E2_STACK", "E3_STACK"], "F_hb": ["E2_HB", "E3_HB"]}
N_REPLICAS = 16


@pytest.fixture(scope="module")
def large(tmp_path_factory):
    w = synth.WORKLOADS["large"]
    d = str(tmp_path_factory.mktemp("large"))
    f = synth.generate(d, "large", w["n_nt"], seed=w["seed"], n_hb_pairs=w["n_hb_pairs"])
    m, cl, k = w["ions"]
    return System.load(f["pdb"], f["bonds"], f["stacks"], f["maxikey"], T=0.59219, box=w["box"], rc=30.0, n_mg=m,
                       n_cl=cl, n_k=k, seed=1, center=500, rng=1)


def _replica(arrays, seed):
    a = dict(arrays)
    a["seed"] = np.array([seed], dtype=np.int64)
    return System.from_arrays(a)


def _terms(system_dict, seed, state, prec, system):
    """Engine and oracle per-term forces and energies at `state` (both with fresh
    rand() streams, so the H-bond Monte Carlo draws the same numbers)."""
    o = Oracle(system_dict, seed=seed)
    if state is not None:
        o.set_state(state)
    o.populate_lists()
    ref = o.terms()
    e = Engine([system], precision=prec)
    if state is not None:
        e.set_state(0, state)
    e.populate_lists()
    got = {}
    for name, mask in TERMS:  # the H-bond term first: its Monte Carlo starts the stream
        got[name] = e.forces(0, mask)
    e.close()
    return ref, got


def test_large_lists_bit_exact(large):
    o = Oracle(large.to_dict(), seed=1)
    o.populate_lists()
    e = Engine([large], precision=PREC_MIXED, full_lists=1)
    e.populate_lists()
    c, dims = e.cells(0)
    oc, od = o.cells()
    assert np.array_equal(dims, od) and np.array_equal(c, oc)
    for which in (0, 1):
        assert np.array_equal(e.pairs(0, which), pair_set(o.pairs(which))), f"list {which}"
    st, ex = e.hb_status(0, o.n_hb, o.n_hba)
    ost, oex = o.hb()
    assert np.array_equal(st, ost) and np.array_equal(ex, oex)


@pytest.mark.parametrize("prec,tol", [(PREC_MIXED, 1e-5), (PREC_FP64, 1e-10)])
def test_large_term_forces_setup_frame(large, prec, tol):
    ref, got = _terms(large.to_dict(), 1, None, prec, large)
    for name, _ in TERMS:
        f, en = got[name]
        want = ref[name]
        if np.linalg.norm(want) == 0:
            continue
        if not (prec == PREC_MIXED and name == "F_stack"):  # native geometry: see the small-system test
            assert rel_err(f, want) <= tol, (name, rel_err(f, want))
        for k in E_TERM[name]:
            assert en[k] == pytest.approx(ref[k], rel=tol, abs=tol * max(1.0, abs(ref[k]))), (name, k)


def _frame_errors(system_dict, seed, state, system):
    o = Oracle(system_dict, seed=seed)
    o.set_state(state)
    o.populate_lists()
    ref = o.terms()
    # the reference's total with the bonded pairs' LJ weighted in the pair sum: its
    # literal sum adds and subtracts that LJ, which reaches 1e17-1e27 kcal/mol/A
    # for a folded 1-3 pair (P-S-B at 1.6 A) and then rounds away the bead's other
    # pair forces
    want = o.net_sr_bonded() + ref["F_lr"] + ref["F_stack"] + ref["F_hb"]
    out = {}
    e = Engine([system], precision=PREC_MIXED)  # fresh rand() stream: the Monte Carlo draws the oracle's numbers
    e.set_state(0, state)
    e.populate_lists()
    e.deterministic_forces()
    out["F_total"] = rel_err(e.current_forces(0), want)
    e.close()
    e = Engine([system], precision=PREC_MIXED)
    e.set_state(0, state)
    e.populate_lists()
    eerr = 0.0
    for name, mask in TERMS:
        if name in ("F_sr", "F_bonded"):
            continue
        f, en = e.forces(0, mask)
        if np.linalg.norm(ref[name]) > 0:
            out[name] = rel_err(f, ref[name])
        for k in E_TERM[name]:
            eerr = max(eerr, abs(en[k] - ref[k]) / max(1.0, abs(ref[k])))
    e.close()
    out["energies"] = eerr
    return out


def test_large_batch_forces_on_100_frames(large):
    """16 replicas run batched (mixed precision); 100 frames taken from the run
    (every replica every 100 steps) are each evaluated by the engine and by the
    FP64 oracle."""
    base = large.to_dict()
    seeds = list(range(1, N_REPLICAS + 1))
    reps = [_replica(base, s) for s in seeds]
    batch = Engine(reps, precision=PREC_MIXED)
    batch.populate_lists()
    frames = []
    while len(frames) < 100:
        batch.step(100)
        batch.sync()
        sts = batch.get_states()
        off = 0
        for r in range(N_REPLICAS):
            n = batch.n[r]
            frames.append((r, {k: sts[k][off:off + n].copy() for k in STATE_NAMES}))
            off += n
    batch.close()
    worst = {}
    for r, st in frames[:100]:
        d = dict(base, seed=np.array([seeds[r]], dtype=np.int64))
        for k, v in _frame_errors(d, seeds[r], st, reps[r]).items():
            worst[k] = max(worst.get(k, 0.0), v)
    print("largest relative error over 100 frames:", ", ".join(f"{k} {v:.2e}" for k, v in worst.items()))
    for k, v in worst.items():
        assert v <= 1e-5, (k, v)
