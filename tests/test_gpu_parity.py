"""GPU parity through the C ABI against the FP64 CPU oracle, on the same systems
(loaded once by the product loader, whose output is pinned to the reference).

Tolerances, stated per check:
  * cell assignments, SR/LR pair sets, H-bond candidate status: bit-exact;
  * per-term forces, mixed precision: ||F_gpu - F_oracle|| / ||F_oracle|| <= 1e-5
    and max_i |F_gpu,i - F_oracle,i| <= 1e-5 * max_i |F_oracle,i|;
  * per-term forces, FP64 mode: relative error <= 1e-10;
  * energies: relative 1e-5 (mixed), 1e-10 (FP64).
"""
import os
import sys

import numpy as np
import pytest

from oracle_bridge import Oracle
from systems import CASES, golden_inputs, load, pair_set, rel_err, stiffness_atol
from tis_gb300 import (PREC_FP64, PREC_MIXED, NOISE_OFF, NOISE_REFERENCE, TERM_BONDED, TERM_HB, TERM_LR, TERM_SR,
                       TERM_STACK, Engine, TisError)

pytestmark = pytest.mark.gpu

TERMS = [("F_sr", TERM_SR), ("F_lr", TERM_LR), ("F_bonded", TERM_BONDED), ("F_stack", TERM_STACK), ("F_hb", TERM_HB)]
E_TERM = {"F_sr": ["E_lj", "E_coul_sr"], "F_lr": ["E_coul_lr"], "F_bonded": ["E_bond", "E_angle", "E_excl"],
          "F_stack": ["E2_STACK", "E3_STACK"], "F_hb": ["E2_HB", "E3_HB"]}
PRECS = [("mixed", PREC_MIXED, 1e-5), ("fp64", PREC_FP64, 1e-10)]


@pytest.fixture(scope="module")
def systems(synth_dir):
    return {"small": load(golden_inputs(), "small"), "central": load(synth_dir["central"], "central")}


def _oracle(sysobj, noise=True, seed=3):
    return Oracle(sysobj.to_dict(), seed=seed, noise=noise)


@pytest.mark.parametrize("prec_name,prec,tol", PRECS)
@pytest.mark.parametrize("case", ["small", "central"])
def test_lists_bit_exact(systems, case, prec_name, prec, tol):
    s = systems[case]
    o = _oracle(s)
    o.populate_lists()
    e = Engine([s], precision=prec, full_lists=1)
    e.populate_lists()
    c, dims = e.cells(0)
    oc, od = o.cells()
    assert np.array_equal(dims, od)
    assert np.array_equal(c, oc)
    for which in (0, 1):
        assert np.array_equal(e.pairs(0, which), pair_set(o.pairs(which))), f"list {which}"
    st, ex = e.hb_status(0, o.n_hb, o.n_hba)
    ost, oex = o.hb()
    assert np.array_equal(st, ost)
    assert np.array_equal(ex, oex)


def _d_lj(sd, ti, tj):
    """D_LJ per type pair (E:2918-2926): 3.2 A among RNA beads, else R_i + R_j."""
    if ti <= 6 and tj <= 6:
        return 3.2
    return sd["rlj"][ti - 1] + sd["rlj"][tj - 1]


@pytest.mark.parametrize("case", ["small", "central"])
def test_pruned_sr_list_keeps_every_interacting_pair(systems, case):
    """The step's SR list (full_lists=0) is the reference's SR set minus pairs with
    a sugar or base bead that lie beyond their LJ range plus the skin, which can
    exert no force before the next rebuild."""
    s = systems[case]
    sd = s.to_dict()
    o = _oracle(s)
    o.populate_lists()
    full = pair_set(o.pairs(0))
    e = Engine([s])
    e.populate_lists()
    pruned = e.pairs(0, 0)
    fset = set(map(tuple, full))
    assert all(tuple(pq) in fset for pq in pruned)
    pset = set(map(tuple, pruned))
    X = np.stack([sd["x"], sd["y"], sd["z"]], 1)
    L = sd["box"]
    kind, typ = sd["kind"], sd["type"]
    need = 0
    for i, j in full:
        charged = kind[i] not in (1, 2) and kind[j] not in (1, 2)
        dv = X[i] - X[j]
        dv -= L * np.round(dv / L)
        r = np.sqrt(dv @ dv)
        if charged or r < (_d_lj(sd, typ[i], typ[j]) + 3.0) * (1 - 1e-4):
            need += 1
            assert (i, j) in pset, (i, j, r)
    assert len(pruned) < len(full) and len(pruned) >= need


def _frame(s, case, frame):
    """The set-up state, or a thermalized frame: 300 oracle steps later."""
    if frame == "initial":
        return None
    o = _oracle(s)
    o.populate_lists()
    o.step(300)
    return o.get_state()


@pytest.mark.parametrize("prec_name,prec,tol", PRECS)
@pytest.mark.parametrize("frame", ["thermal", "initial"])
@pytest.mark.parametrize("case", ["small", "central"])
def test_term_forces_and_energies(systems, case, frame, prec_name, prec, tol):
    """Per-term forces and energies on identical coordinates: ||dF|| / ||F|| and
    max |dF_i| / max |F_i| within tol, with, in mixed precision, the per-bead FP32
    allowance of stiffness_atol added (it matters on the set-up frame, where the
    stacks' and native H-bonds' true forces vanish)."""
    s = systems[case]
    st = _frame(s, case, frame)
    o = _oracle(s)
    if st is not None:
        o.set_state(st)
    o.populate_lists()
    ref = o.terms()
    atol = stiffness_atol(s.to_dict()) if prec == PREC_MIXED else 0.0
    report = []
    for name, mask in TERMS:
        e = Engine([s], precision=prec)  # fresh: the H-bond term consumes Monte Carlo draws
        if st is not None:
            e.set_state(0, st)
        e.populate_lists()
        f, en = e.forces(0, mask)
        want = ref[name]
        if np.linalg.norm(want) == 0:
            assert np.abs(f).max() < 1e-12, name
            continue
        rel = rel_err(f, want)
        dabs = np.abs(f - want).max()
        fmax = np.abs(want).max()
        report.append(f"{name} rel {rel:.2e} max|dF| {dabs:.2e} (|F|max {fmax:.2e}, atol {atol:.1e})")
        assert dabs <= tol * fmax + atol, (name, dabs, fmax)
        assert np.linalg.norm(f - want) <= tol * np.linalg.norm(want) + atol * np.sqrt(want.size), (name, rel)
        for k in E_TERM[name]:
            assert en[k] == pytest.approx(ref[k], rel=tol, abs=tol * max(1.0, abs(ref[k]))), (name, k)
    print(f"{case} {frame} {prec_name}: " + "; ".join(report))
    e = Engine([s], precision=prec)
    if st is not None:
        e.set_state(0, st)
    e.populate_lists()
    f, en = e.forces(0, TERM_SR | TERM_LR | TERM_BONDED | TERM_STACK | TERM_HB)
    total = sum(ref[n] for n, _ in TERMS)
    assert np.abs(f - total).max() <= tol * np.abs(total).max() + atol
    assert np.linalg.norm(f - total) <= tol * np.linalg.norm(total) + atol * np.sqrt(total.size)
    assert en["Rg"] == pytest.approx(ref["Rg"], rel=1e-12)


@pytest.mark.parametrize("prec_name,prec,tol", PRECS)
@pytest.mark.parametrize("case", ["small", "central"])
def test_hot_path_total_force(systems, case, prec_name, prec, tol):
    """tis_deterministic_forces (the step's force pass, which leaves bonded pairs'
    LJ out of the SR sum instead of adding and subtracting it) gives the
    reference's total deterministic force (E:2524-2586) on a thermalized frame."""
    s = systems[case]
    st = _frame(s, case, "thermal")
    o = _oracle(s)
    o.set_state(st)
    o.populate_lists()
    ref = o.terms()
    want = sum(ref[n] for n, _ in TERMS)
    e = Engine([s], precision=prec)
    e.set_state(0, st)
    e.populate_lists()
    e.deterministic_forces()
    f = e.current_forces(0)
    assert rel_err(f, want) <= tol, rel_err(f, want)
    assert np.abs(f - want).max() <= tol * np.abs(want).max()


def test_bench_system_runs_stably():
    """The batched benchmark's replicas (346-nt chain, Mg 0 and 20 mM): 2000 mixed
    steps without a flagged force, and the first 100 steps track the oracle."""
    import tempfile
    import bench
    d = tempfile.mkdtemp()
    files = bench.make_inputs(d)
    specs = bench.replica_specs()
    sys_ = bench.load_systems(files, [specs[0], specs[-1]])
    e = Engine(sys_)
    e.populate_lists()
    o = Oracle(sys_[0].to_dict(), seed=specs[0]["seed"])
    o.populate_lists()
    e.step(100)
    o.step(100)
    e.sync()
    d100 = np.abs(_positions(e.get_state(0)) - _positions(o.get_state())).max()
    assert d100 < 1e-3, d100
    e.step(1900)
    e.sync()


def _positions(st):
    return np.stack([st["x"], st["y"], st["z"]], 1)


@pytest.mark.parametrize("prec_name,prec,tol_pos", [("fp64", PREC_FP64, 1e-7), ("mixed", PREC_MIXED, 1e-3)])
def test_noise_free_trajectory_tracks_oracle(systems, prec_name, prec, tol_pos):
    """1000 noise-free steps of the small system (H-bond Monte Carlo on the shared
    stream): max position deviation from the FP64 oracle stays below tol_pos A."""
    s = systems["small"]
    o = _oracle(s, noise=False)
    o.populate_lists()
    e = Engine([s], precision=prec, noise=NOISE_OFF)
    e.populate_lists()
    dev = []
    for k in range(10):
        o.step(100)
        e.step(100)
        e.sync()
        d = np.abs(_positions(e.get_state(0)) - _positions(o.get_state())).max()
        dev.append(d)
    print(f"{prec_name} max |dx| every 100 steps:", " ".join(f"{d:.2e}" for d in dev))
    assert max(dev) < tol_pos
    assert e.counters(0)[2] == o.draws()


# Per-checkpoint bounds (A) of the 10^4-step divergence curves, every 1000 steps:
# about three times the measured curves, made non-decreasing.  The FP64 path adds
# its forces with atomics in arbitrary order, so its curve varies from run to run
# (two runs: 6e-10, 6e-9, 5e-8, 1e-7, 2e-6, 1e-5, 9e-6, 4e-5, 8e-4, 5e-3 and 7e-10,
# 9e-9, 8e-8, 7e-7, 9e-6, 5e-5, 3e-5, 3e-5, 2e-4, 2e-3): three times the larger;
# the mixed path is deterministic (fixed-point sums): 8e-6, 1e-5, 2e-5, 1.5e-4,
# 1.9e-3, 2.4e-2, 1.5e-2, 1.7e-2, 9.2e-2, 6.7e-2.
ENVELOPE_10K = {
    "fp64": [2e-9, 3e-8, 3e-7, 2e-6, 3e-5, 1.6e-4, 1.6e-4, 1.6e-4, 2.5e-3, 2e-2],
    "mixed": [2.5e-5, 4e-5, 7e-5, 5e-4, 6e-3, 7.5e-2, 7.5e-2, 7.5e-2, 0.28, 0.28],
}


@pytest.mark.parametrize("prec_name,prec,tol_pos", [("fp64", PREC_FP64, 2e-2), ("mixed", PREC_MIXED, 0.28)])
def test_noise_free_trajectory_10k_steps(systems, prec_name, prec, tol_pos):
    """10^4 noise-free steps of the small system against the FP64 oracle: the
    divergence curve (max position deviation every 1000 steps) is printed and held
    to ENVELOPE_10K checkpoint by checkpoint.  Any difference grows with the
    dynamics' own sensitivity (about tenfold per 1000 steps): the FP64 path, which
    differs from the oracle only in the order of its force sums (1e-13 A after 100
    steps), reaches ~5e-3 A at 10^4 steps; mixed precision, which rounds each pair
    force to FP32, levels off at a few 1e-2 A."""
    s = systems["small"]
    o = _oracle(s, noise=False)
    o.populate_lists()
    e = Engine([s], precision=prec, noise=NOISE_OFF)
    e.populate_lists()
    dev = []
    for k in range(10):
        o.step(1000)
        e.step(1000)
        e.sync()
        dev.append(np.abs(_positions(e.get_state(0)) - _positions(o.get_state())).max())
    print(f"{prec_name} max |dx| every 1000 steps:", " ".join(f"{d:.2e}" for d in dev))
    for k, (d, bound) in enumerate(zip(dev, ENVELOPE_10K[prec_name])):
        assert d < bound, (k, d, bound)
    assert max(dev) < tol_pos


@pytest.mark.parametrize("prec_name,prec,tol_pos", [("fp64", PREC_FP64, 1e-7), ("mixed", PREC_MIXED, 1e-3)])
def test_stochastic_trajectory_tracks_oracle(systems, prec_name, prec, tol_pos):
    """Langevin noise and Monte Carlo from the shared Philox stream: 200 steps."""
    s = systems["small"]
    o = _oracle(s, noise=True)
    o.populate_lists()
    e = Engine([s], precision=prec, noise=NOISE_REFERENCE)
    e.populate_lists()
    o.step(200)
    e.step(200)
    e.sync()
    d = np.abs(_positions(e.get_state(0)) - _positions(o.get_state())).max()
    print(f"{prec_name} stochastic 200 steps max |dx| = {d:.2e}")
    assert d < tol_pos
    assert e.counters(0)[2] == o.draws()
    np.testing.assert_allclose(e.energies(0), o.last_energies(), rtol=1e-3 if prec == PREC_MIXED else 1e-8, atol=1e-3)


def test_batch_equals_single_bitwise(synth_dir):
    """Replicas with different ion numbers, temperatures and seeds advance in one
    batch exactly as each does alone (fixed-point sums are order-independent)."""
    f = synth_dir["small"]
    specs = [dict(seed=3), dict(seed=5, n_mg=20, n_cl=281, n_k=317, T=0.62), dict(seed=9, n_mg=0, n_cl=241, n_k=317)]
    sys_ = [load(f, "small", **sp) for sp in specs]
    batch = Engine(sys_)
    batch.populate_lists()
    batch.step(300)
    batch.sync()
    for r, s in enumerate(sys_):
        one = Engine([s])
        one.populate_lists()
        one.step(300)
        one.sync()
        a, b = batch.get_state(r), one.get_state(0)
        for k in a:
            assert np.array_equal(a[k], b[k]), (r, k)
        assert batch.counters(r) == one.counters(0)


def test_replica_groups_equal_one_group_bitwise(synth_dir):
    """Splitting a handle's replicas into concurrently running groups changes no
    result: the fused graph step and the four drop-in calls both match one group."""
    f = synth_dir["small"]
    specs = [dict(seed=3 + 2 * k, n_mg=10 + 2 * k, n_cl=261 + 4 * k, n_k=317) for k in range(5)]
    sys_ = [load(f, "small", **sp) for sp in specs]
    runs = []
    for groups, split in [(1, False), (3, False), (2, True)]:
        e = Engine(sys_, groups=groups, graph_steps=20)
        e.populate_lists()
        if split:
            for _ in range(120):
                e.deterministic_forces()
                e.full_forces()
                e.move_rigid_units()
                e.check_shifts()
        else:
            e.step(120)
        e.sync()
        runs.append(([e.get_state(r) for r in range(len(sys_))], [e.counters(r) for r in range(len(sys_))]))
    for states, counters in runs[1:]:
        assert counters == runs[0][1]
        for r in range(len(sys_)):
            for k in states[r]:
                assert np.array_equal(states[r][k], runs[0][0][r][k]), (r, k)


def test_batched_state_calls_equal_per_replica_calls(synth_dir):
    """tis_set_states / tis_get_states / tis_get_all_energies (all replicas, packed
    end to end, one copy per array and group) equal the per-replica calls."""
    f = synth_dir["small"]
    specs = [dict(seed=3 + 2 * k, n_mg=10 + 2 * k, n_cl=261 + 4 * k, n_k=317) for k in range(5)]
    sys_ = [load(f, "small", **sp) for sp in specs]
    e = Engine(sys_, groups=2)
    e.populate_lists()
    e.step(60)
    e.sync()
    packed = e.get_states()
    per = [e.get_state(r) for r in range(len(sys_))]
    for k in per[0]:
        assert np.array_equal(packed[k], np.concatenate([p[k] for p in per])), k
    en = e.all_energies()
    for r in range(len(sys_)):
        assert np.array_equal(en[r], e.energies(r)), r
    mod = {k: v.copy() for k, v in packed.items()}
    mod["vx"] *= 0.5
    batched = Engine(sys_, groups=3)
    batched.set_states(mod)
    single = Engine(sys_, groups=1)
    off = 0
    for r in range(len(sys_)):
        n = single.n[r]
        single.set_state(r, {k: mod[k][off:off + n] for k in mod})
        off += n
    for eng in (batched, single):
        eng.populate_lists()
        eng.step(40)
        eng.sync()
    a, b = batched.get_states(), single.get_states()
    for k in a:
        assert np.array_equal(a[k], b[k]), k


def test_split_calls_and_graph_equal_fused_step(systems):
    """The four drop-in calls (deterministic_forces, full_forces, move_rigid_units,
    check_shifts), the fused step and the captured graph give identical states."""
    s = systems["small"]
    runs = []
    for mode in ["split", "direct", "graph", "captured"]:
        e = Engine([s], use_graph=1 if mode == "graph" else 0, graph_steps=20)
        e.populate_lists()
        if mode == "captured":  # tis_capture_graph: a 25-step graph replayed 4 times
            e.capture_graph(25)
            e.step(100)
        elif mode == "split":
            for _ in range(100):
                e.deterministic_forces()
                e.full_forces()
                e.move_rigid_units()
                e.check_shifts()
        else:
            e.step(100)
        e.sync()
        runs.append(e.get_state(0))
    for k in runs[0]:
        assert np.array_equal(runs[0][k], runs[1][k]), k
        assert np.array_equal(runs[1][k], runs[2][k]), k
        assert np.array_equal(runs[1][k], runs[3][k]), k


def test_nonfinite_state_is_reported(systems):
    s = systems["small"]
    e = Engine([s])
    st = e.get_state(0)
    st["vx"][5] = np.inf
    e.set_state(0, st)
    e.populate_lists()
    e.step(2)
    with pytest.raises(TisError) as err:
        e.sync()
    assert err.value.code == 6


def test_small_capacity_grows_at_list_build(systems):
    s = systems["central"]
    e = Engine([s], cap_sr=8, cap_lr=8, full_lists=1)
    e.populate_lists()  # overflows, grows, rebuilds
    o = _oracle(s)
    o.populate_lists()
    assert np.array_equal(e.pairs(0, 0), pair_set(o.pairs(0)))
