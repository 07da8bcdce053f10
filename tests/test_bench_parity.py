"""Per-term parity on the batched workload's own replicas (the 64-replica Mg sweep
of the 346-nt chain in a 350 A box, rc 30 A): replicas 0, 31 and 63 (0, 9.8 and
20 mM Mg; 0, 254 and 516 Mg2+, 4.6k-6.1k particles), on the set-up frame and on
the frame reached after 1000 steps of the three run as one mixed-precision batch.

Checked against the FP64 oracle on identical coordinates:
  * cell assignments and the full SR / LR pair sets: bit-exact, with the pairs
    lying within 0.1% of a list radius counted (the FP32 decision band is
    exercised on these dense lists);
  * per-term forces, mixed precision: ||dF|| / ||F|| <= 1e-5 and, per bead,
    |dF_i| <= 1e-5 |F|_max + atol, where atol (systems.stiffness_atol, 2.1e-4
    kcal/mol/A here) covers FP32 rounding of a term whose true force vanishes (a
    stack or H-bond at its native geometry on the set-up frame);
  * per-term energies: relative 1e-5;
  * FP64 mode: relative 1e-10 per term.
"""
import numpy as np
import pytest

from oracle_bridge import Oracle
from systems import pair_set, rel_err, stiffness_atol
from tis_gb300 import (PREC_FP64, PREC_MIXED, TERM_BONDED, TERM_HB, TERM_LR, TERM_SR, TERM_STACK, Engine)

pytestmark = pytest.mark.gpu

TERMS = [("F_sr", TERM_SR), ("F_lr", TERM_LR), ("F_bonded", TERM_BONDED), ("F_stack", TERM_STACK), ("F_hb", TERM_HB)]
E_TERM = {"F_sr": ["E_lj", "E_coul_sr"], "F_lr": ["E_coul_lr"], "F_bonded": ["E_bond", "E_angle", "E_excl"],
          "F_stack": ["E2_STACK", "E3_STACK"], "F_hb": ["E2_HB", "E3_HB"]}
PICK = [0, 31, 63]


@pytest.fixture(scope="module")
def bench_replicas(tmp_path_factory):
    import bench
    files = bench.make_inputs(str(tmp_path_factory.mktemp("bench")))
    specs = bench.replica_specs()
    systems = bench.load_systems(files, [specs[r] for r in PICK])
    # the frame after 1000 batched mixed-precision steps of the three together
    e = Engine(systems, precision=PREC_MIXED)
    e.populate_lists()
    e.step(1000)
    e.sync()
    later = [e.get_state(k) for k in range(len(PICK))]
    e.close()
    return systems, [specs[r] for r in PICK], later


def _band_counts(o, sd, which, radius):
    p = o.pairs(which).reshape(-1, 2)
    X = np.stack([sd["x"], sd["y"], sd["z"]], 1)
    L = np.asarray(sd["box"], dtype=np.float64)
    dv = X[p[:, 0]] - X[p[:, 1]]
    dv -= L * np.round(dv / L)
    r = np.sqrt((dv * dv).sum(1))
    return int((np.abs(r / radius - 1.0) < 1e-3).sum())


@pytest.mark.parametrize("frame", ["setup", "after_1000_batched"])
@pytest.mark.parametrize("k", range(len(PICK)))
def test_bench_replica_lists_bit_exact(bench_replicas, k, frame):
    systems, specs, later = bench_replicas
    s = systems[k]
    sd = s.to_dict()
    st = None if frame == "setup" else later[k]
    if st is not None:
        sd = dict(sd, **{n: st[n] for n in ("x", "y", "z")})
    o = Oracle(s.to_dict(), seed=specs[k]["seed"])
    if st is not None:
        o.set_state(st)
    o.populate_lists()
    e = Engine([s], precision=PREC_MIXED, full_lists=1)
    if st is not None:
        e.set_state(0, st)
    e.populate_lists()
    c, dims = e.cells(0)
    oc, od = o.cells()
    assert np.array_equal(dims, od) and np.array_equal(c, oc)
    near = []
    for which, radius in ((0, 15.0), (1, 33.0)):
        got = e.pairs(0, which)
        want = pair_set(o.pairs(which))
        assert got.shape == want.shape and np.array_equal(got, want), (PICK[k], frame, which)
        near.append(_band_counts(o, sd, which, radius))
    print(f"replica {PICK[k]} {frame}: {len(e.pairs(0, 0))} SR / {len(e.pairs(0, 1))} LR pairs, "
          f"{near[0]} / {near[1]} within 0.1% of 15 / 33 A")
    st_h, ex_h = e.hb_status(0, o.n_hb, o.n_hba)
    ost, oex = o.hb()
    assert np.array_equal(st_h, ost) and np.array_equal(ex_h, oex)


@pytest.mark.parametrize("prec_name,prec,tol", [("mixed", PREC_MIXED, 1e-5), ("fp64", PREC_FP64, 1e-10)])
@pytest.mark.parametrize("frame", ["setup", "after_1000_batched"])
@pytest.mark.parametrize("k", range(len(PICK)))
def test_bench_replica_term_forces(bench_replicas, k, frame, prec_name, prec, tol):
    systems, specs, later = bench_replicas
    s = systems[k]
    st = None if frame == "setup" else later[k]
    o = Oracle(s.to_dict(), seed=specs[k]["seed"])
    if st is not None:
        o.set_state(st)
    o.populate_lists()
    ref = o.terms()
    atol = stiffness_atol(s.to_dict()) if prec == PREC_MIXED else 0.0
    report = []
    total = np.zeros_like(ref["F_sr"])
    for name, mask in TERMS:
        e = Engine([s], precision=prec)  # fresh: the H-bond term consumes Monte Carlo draws
        if st is not None:
            e.set_state(0, st)
        e.populate_lists()
        f, en = e.forces(0, mask)
        e.close()
        want = ref[name]
        total += want
        if np.linalg.norm(want) == 0:
            assert np.abs(f).max() < 1e-12, name
            continue
        rel = rel_err(f, want)
        fmax = np.abs(want).max()
        dabs = np.abs(f - want).max()
        report.append(f"{name} rel {rel:.1e} max|dF| {dabs:.1e} (|F|max {fmax:.1e})")
        assert dabs <= tol * fmax + atol, (name, dabs, tol * fmax + atol)
        # the norm criterion, with the same absolute allowance spread over the beads
        assert np.linalg.norm(f - want) <= tol * np.linalg.norm(want) + atol * np.sqrt(want.size), (name, rel)
        for kk in E_TERM[name]:
            assert en[kk] == pytest.approx(ref[kk], rel=tol, abs=tol * max(1.0, abs(ref[kk]))), (name, kk)
    print(f"replica {PICK[k]} {frame} {prec_name}: " + "; ".join(report))
    e = Engine([s], precision=prec)
    if st is not None:
        e.set_state(0, st)
    e.populate_lists()
    f, en = e.forces(0, TERM_SR | TERM_LR | TERM_BONDED | TERM_STACK | TERM_HB)
    assert np.abs(f - total).max() <= tol * np.abs(total).max() + atol
    assert en["Rg"] == pytest.approx(ref["Rg"], rel=1e-12)


def test_bench_replicas_hot_path_total_force(bench_replicas):
    """The step's own force pass (bonded pairs' LJ left out of the SR sum) on the
    three replicas after 1000 batched steps, all on one handle as in the bench:
    the reference's total deterministic force within 1e-5."""
    systems, specs, later = bench_replicas
    e = Engine(systems, precision=PREC_MIXED)
    for k, st in enumerate(later):
        e.set_state(k, st)
    e.populate_lists()
    e.deterministic_forces()
    for k, s in enumerate(systems):
        o = Oracle(s.to_dict(), seed=specs[k]["seed"])
        o.set_state(later[k])
        o.populate_lists()
        ref = o.terms()
        want = sum(ref[n] for n, _ in TERMS)
        f = e.current_forces(k)
        assert rel_err(f, want) <= 1e-5, (PICK[k], rel_err(f, want))
        assert np.abs(f - want).max() <= 1e-5 * np.abs(want).max() + stiffness_atol(s.to_dict())
