"""The C oracle is pinned to the reference engine: against committed golden
fixtures made by the reference itself (tests/golden/make_golden.py), and against
the live reference when its sources are present.  CPU only."""
import ctypes as C
import os

import numpy as np
import pytest

from oracle_bridge import Oracle, ensure_oracle, ref_available, run_ref, REF_SRC_DIR
from systems import CASES, pair_set, read_golden, ref_kwargs, rel_err
from tis_gb300 import tisb

# Random123 known-answer vectors for philox4x32_10
PHILOX_KAT = [
    ((0, 0, 0, 0), (0, 0), (0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8)),
    ((0xffffffff,) * 4, (0xffffffff, 0xffffffff), (0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd)),
    ((0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344), (0xa4093822, 0x299f31d0),
     (0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1)),
]


def test_oracle_philox_known_answers():
    lib = C.CDLL(ensure_oracle())
    lib.tis_o_philox_word.restype = C.c_uint32
    lib.tis_o_philox_word.argtypes = [C.c_uint32] * 6 + [C.c_int]
    for ctr, key, want in PHILOX_KAT:
        got = tuple(lib.tis_o_philox_word(*ctr, *key, lane) for lane in range(4))
        assert got == want


@pytest.fixture(scope="module")
def golden_small():
    return (read_golden("small_ref_system.bin"), read_golden("small_ref_lists.bin"),
            read_golden("small_ref_terms.bin"))


def test_oracle_lists_bit_exact(golden_small):
    s, L, _ = golden_small
    o = Oracle(s, seed=3)
    o.populate_lists()
    cell, dims = o.cells()
    assert np.array_equal(dims, L["cells_dim"])
    assert np.array_equal(cell, L["cell"])
    # the oracle visits cells exactly as populate_lists does: same pairs, same order
    assert np.array_equal(o.pairs(0), L["sr_pairs"])
    assert np.array_equal(o.pairs(1), L["lr_pairs"])
    st, ex = o.hb()
    assert np.array_equal(st, L["hb_status"])
    assert np.array_equal(ex, L["hb_excess"])


def test_oracle_terms_match_reference(golden_small):
    s, _, T = golden_small
    o = Oracle(s, seed=3)
    o.populate_lists()
    t = o.terms()
    for k in ["F_sr", "F_lr", "F_bonded", "F_stack", "F_hb"]:
        assert rel_err(t[k], T[k]) < 1e-12, k
    for k in ["E_lj", "E_coul_sr", "E_coul_lr", "E_bond", "E_angle", "E_excl", "E2_STACK", "E3_STACK", "E2_HB",
              "E3_HB", "Rg"]:
        assert t[k] == pytest.approx(T[k][0], rel=1e-12, abs=1e-12), k
    assert np.array_equal(t["st_status"], T["st_status"])


@pytest.mark.parametrize("fixture,noise", [("small_ref_traj.bin", True), ("small_ref_quiet.bin", False)])
def test_oracle_tracks_reference_trajectory(golden_small, fixture, noise):
    """300 steps with the H-bond Monte Carlo (and the noise) drawing from the
    shared Philox stream: the oracle follows the reference to rounding."""
    s = golden_small[0]
    R = read_golden(fixture)
    o = Oracle(s, seed=3, noise=noise)
    o.populate_lists()
    for k in range(1, 7):
        o.step(50)
        st = o.get_state()
        pos = np.stack([st["x"], st["y"], st["z"]], 1).ravel()
        assert np.abs(pos - R[f"pos_{50 * k}"]).max() < 1e-8
        np.testing.assert_allclose(o.last_energies(), R["energies"][5 * (k - 1): 5 * k], rtol=1e-9, atol=1e-9)
    assert o.draws() == int(R["draws"][0])
    assert o.rebuilds() - 1 == len(R["rebuild_steps"])


needs_ref = pytest.mark.skipif(not ref_available(), reason="oracle/_ref not built (reference sources absent)")


@needs_ref
def test_oracle_matches_live_reference_central(synth_dir, tmp_path):
    f = synth_dir["central"]
    o_ = run_ref(f, str(tmp_path), "c", extra=("export-system", "lists", "terms"), **ref_kwargs("central"))
    s, L, T = tisb.read(o_["export-system"]), tisb.read(o_["lists"]), tisb.read(o_["terms"])
    o = Oracle(s, seed=3)
    o.populate_lists()
    assert np.array_equal(o.cells()[0], L["cell"])
    assert np.array_equal(o.pairs(0), L["sr_pairs"])
    assert np.array_equal(o.pairs(1), L["lr_pairs"])
    t = o.terms()
    for k in ["F_sr", "F_lr", "F_bonded", "F_stack", "F_hb"]:
        assert rel_err(t[k], T[k]) < 1e-12, k


@needs_ref
def test_oracle_matches_live_reference_large(tmp_path):
    """The large system (1500-nt chain, 600 A box, 1300 Mg / 22100 Cl / 21000 K,
    48,899 particles): the reference's own engine and the oracle give the same
    cells, SR/LR pair sets and forces."""
    from tis_gb300 import synth
    w = synth.WORKLOADS["large"]
    f = synth.generate(str(tmp_path), "large", w["n_nt"], seed=w["seed"], n_hb_pairs=w["n_hb_pairs"])
    m, cl, k = w["ions"]
    o_ = run_ref(f, str(tmp_path), "L", extra=("export-system", "lists", "terms"), box=w["box"], rc=30.0,
                 T=0.59219, nMg=m, nCl=cl, nK=k, seed=1, center=500, rng="philox")
    s, L, T = tisb.read(o_["export-system"]), tisb.read(o_["lists"]), tisb.read(o_["terms"])
    o = Oracle(s, seed=1)
    o.populate_lists()
    assert np.array_equal(o.cells()[0], L["cell"])
    assert np.array_equal(o.pairs(0), L["sr_pairs"])
    assert np.array_equal(o.pairs(1), L["lr_pairs"])
    t = o.terms()
    for k in ["F_sr", "F_lr", "F_bonded", "F_stack", "F_hb"]:
        assert rel_err(t[k], T[k]) < 1e-12, k


SHIPPED = os.path.join(REF_SRC_DIR, "src")


@needs_ref
@pytest.mark.skipif(not os.path.isdir(SHIPPED), reason="reference data files absent")
def test_oracle_matches_live_reference_shipped_16S(tmp_path):
    """The shipped 16S central domain (3659 particles, 22637 H-bond candidates)."""
    f = dict(pdb=os.path.join(SHIPPED, "16SCD.pdb"), bonds=os.path.join(SHIPPED, "16SCD_16SCD_unprocessed_bonds.dat"),
             stacks=os.path.join(SHIPPED, "16SCD_16SCD_unprocessed_stacks.dat"),
             maxikey=os.path.join(SHIPPED, "MAXIKEY_Mg_Cl_K.dat"))
    kw = dict(T=0.615, cMg=0.005, cK=0.05, seed=1, rng="philox")
    o_ = run_ref(f, str(tmp_path), "s", extra=("export-system", "lists", "terms"), **kw)
    s, L, T = tisb.read(o_["export-system"]), tisb.read(o_["lists"]), tisb.read(o_["terms"])
    o = Oracle(s, seed=1, rc=50.0)
    o.populate_lists()
    assert np.array_equal(o.pairs(0), L["sr_pairs"])
    assert np.array_equal(o.pairs(1), L["lr_pairs"])
    st, ex = o.hb()
    assert np.array_equal(st, L["hb_status"]) and np.array_equal(ex, L["hb_excess"])
    t = o.terms()
    for k in ["F_sr", "F_lr", "F_bonded", "F_stack", "F_hb"]:
        assert rel_err(t[k], T[k]) < 1e-12, k
    o_ = run_ref(f, str(tmp_path), "s", extra=("traj", "--steps", "100", "--every", "50"), **kw)
    R = tisb.read(o_["traj"])
    o = Oracle(s, seed=1, rc=50.0)
    o.populate_lists()
    o.step(100)
    st = o.get_state()
    pos = np.stack([st["x"], st["y"], st["z"]], 1).ravel()
    assert np.abs(pos - R["pos_100"]).max() < 1e-8
    assert o.draws() == int(R["draws"][0])
