"""The host loader (tis_system_load) reproduces the reference's set-up: same
topology arrays and the same initial state, bit for bit.  CPU only."""
import json
import os
import shutil

import numpy as np
import pytest

from oracle_bridge import REF_SRC_DIR, ref_available, run_ref
from systems import CASES, golden_inputs, load, read_golden, ref_kwargs
from tis_gb300 import System, TisError, synth, tisb


def _compare(mine, ref):
    bad = []
    for k, v in ref.items():
        m = mine.get(k)
        if m is None or m.shape != v.shape or not np.array_equal(m.astype(v.dtype), v):
            bad.append(k)
    return bad


def test_loader_matches_reference_golden():
    s = load(golden_inputs(), "small")
    assert _compare(s.to_dict(), read_golden("small_ref_system.bin")) == []


@pytest.mark.skipif(not ref_available(), reason="oracle/_ref not built (reference sources absent)")
@pytest.mark.parametrize("rng", ["glibc", "philox"])
def test_loader_matches_live_reference_central(synth_dir, tmp_path, rng):
    f = synth_dir["central"]
    o = run_ref(f, str(tmp_path), "c", extra=("export-system",), **ref_kwargs("central", rng=rng))
    s = load(f, "central", rng=1 if rng == "philox" else 0)
    assert _compare(s.to_dict(), tisb.read(o["export-system"])) == []


SHIPPED = os.path.join(REF_SRC_DIR, "src")


def _shipped():
    return dict(pdb=os.path.join(SHIPPED, "16SCD.pdb"), bonds=os.path.join(SHIPPED, "16SCD_16SCD_unprocessed_bonds.dat"),
                stacks=os.path.join(SHIPPED, "16SCD_16SCD_unprocessed_stacks.dat"),
                maxikey=os.path.join(SHIPPED, "MAXIKEY_Mg_Cl_K.dat"))


@pytest.mark.skipif(not os.path.isdir(SHIPPED), reason="reference data files absent")
def test_loader_shipped_16S_against_reference_pins(golden_dir):
    """The reference's own topology dump fragments (make_ninfo/*.edit.ninfo) pin the
    H-bond and tertiary-stack parameters of the shipped system."""
    pins = json.load(open(os.path.join(golden_dir, "reference_pins.json")))
    f = _shipped()
    s = System.load(f["pdb"], f["bonds"], f["stacks"], f["maxikey"], T=0.615, c_mg=0.005, c_k=0.05, seed=1)
    hbE, hbn = s["hb_E"], s["hb_native"].reshape(-1, 6)
    assert len(hbE) == pins["hb_rows"]
    for k, row in enumerate(pins["hb_first_rows"]):
        assert round(hbE[k], 3) == pytest.approx(row["eps"], abs=1e-9)
        assert round(hbn[k, 0], 2) == pytest.approx(row["r0"], abs=1e-9)
    stE, stn = s["st3_E"], s["st3_native"].reshape(-1, 6)
    assert len(stE) == pins["tbs_rows"]
    for k, row in enumerate(pins["tbs_first_rows"]):
        assert stE[k] == pytest.approx(row["eps"])
        assert round(stn[k, 0], 2) == pytest.approx(row["r0"], abs=1e-9)
    assert list(s["n_ions"]) == [129, 1203, 1290]
    assert int(s["n_particles"][0]) == 3659


@pytest.mark.skipif(not (ref_available() and os.path.isdir(SHIPPED)), reason="reference absent")
def test_loader_shipped_16S_matches_live_reference(tmp_path):
    f = _shipped()
    o = run_ref(f, str(tmp_path), "s", extra=("export-system",), T=0.615, cMg=0.005, cK=0.05, seed=1)
    s = System.load(f["pdb"], f["bonds"], f["stacks"], f["maxikey"], T=0.615, c_mg=0.005, c_k=0.05, seed=1)
    assert _compare(s.to_dict(), tisb.read(o["export-system"])) == []


def test_ion_count_rule_matches_stored_values(golden_dir):
    """E:6167-6171 against the reference's stored per-[Mg] ion numbers (350 A box,
    50 mM KCl): Mg and K from the bulk concentrations, Cl neutralising."""
    pins = json.load(open(os.path.join(golden_dir, "reference_pins.json")))["ion_counts_350A_50mM_KCl"]
    g = golden_inputs()
    n_entries = int(read_golden("small_ref_system.bin")["n_entries"][0])
    for c in ["0.0", "0.0005", "0.002", "0.005"] + [k for k in list(pins["nMgs"])[::4]]:
        if c not in pins["nMgs"]:
            continue
        s = System.load(g["pdb"], g["bonds"], g["stacks"], g["maxikey"], T=0.615, box=350.0, rc=30.0,
                        c_mg=float(c), c_k=0.05, center=100, seed=2)
        n_mg, n_cl, n_k = (int(v) for v in s["n_ions"])
        assert n_mg == pins["nMgs"][c]
        assert n_k == pins["nKs"][c]
        # the shipped chain has 691 entries; Cl = 2 Mg + K - (entries - 1)/2
        assert pins["nCls"][c] == 2 * pins["nMgs"][c] + pins["nKs"][c] - (691 - 1) // 2
        assert n_cl == 2 * n_mg + n_k - (n_entries - 1) // 2


def test_loader_rejects_bad_inputs(tmp_path):
    g = golden_inputs()
    with pytest.raises(TisError) as e:
        System.load(str(tmp_path / "missing.pdb"), g["bonds"], g["stacks"], g["maxikey"])
    assert e.value.code == 2
    bad = tmp_path / "bonds_nl.dat"
    shutil.copy(g["bonds"], bad)
    with open(bad, "a") as fh:
        fh.write("\n")  # the reference's feof() loop would run once more on stale tokens
    with pytest.raises(TisError) as e:
        System.load(g["pdb"], str(bad), g["stacks"], g["maxikey"], center=100, box=200.0)
    assert e.value.code == 3
    empty = tmp_path / "stacks_empty.dat"
    empty.write_text("")
    with pytest.raises(TisError) as e:
        System.load(g["pdb"], g["bonds"], str(empty), g["maxikey"], center=100, box=200.0)
    assert e.value.code == 3
    with pytest.raises(TisError) as e:
        System.load(g["pdb"], g["bonds"], g["stacks"], g["maxikey"], center=100000, box=200.0)
    assert e.value.code == 1


def test_generator_is_deterministic(tmp_path):
    a = synth.generate(str(tmp_path / "a"), "s", 30, seed=11, n_hb_pairs=5)
    b = synth.generate(str(tmp_path / "b"), "s", 30, seed=11, n_hb_pairs=5)
    for k in ["pdb", "bonds", "stacks"]:
        assert open(a[k]).read() == open(b[k]).read()
    n_nt = 30
    s = System.load(a["pdb"], a["bonds"], a["stacks"], a["maxikey"], center=10, box=200.0, n_mg=2, n_cl=60, n_k=40)
    assert int(s["n_rna"][0]) == 3 * n_nt - 1
    assert len(s["st2_E"]) == n_nt - 3
