"""The topology exporter's three files (CafeMol .ninfo, PSF, coarse-grained PDB)
against the reference's own exporter, analysis/make_ninfo/16SCD_ninfo.cpp,
compiled here unmodified (oracle/build_ref.py) and run on the shipped 16S system
with the flags of its exe.sh: every file byte for byte.  The reference is only
present in the build container, so the pin skips elsewhere; the record counts of
the .ninfo file are checked on the committed 76-nt system everywhere."""
import os
import shutil
import subprocess

import numpy as np
import pytest

import build_ref
from systems import golden_inputs, load
from tis_gb300 import System

REF_ROOT = os.environ.get("TIS_REFERENCE_ROOT", "/root/reference")
SHIPPED = os.path.join(REF_ROOT, "analysis", "make_ninfo")
INPUTS = ["16SCD.pdb", "16SCD_16SCD_unprocessed_bonds.dat", "16SCD_16SCD_unprocessed_stacks.dat",
          "MAXIKEY_Mg_Cl_K.dat"]


@pytest.fixture(scope="module")
def reference_outputs(tmp_path_factory):
    exe = build_ref.build_exporter()
    if exe is None or not all(os.path.isfile(os.path.join(SHIPPED, f)) for f in INPUTS):
        pytest.skip("the reference's exporter and the shipped 16S system are not available here")
    d = tmp_path_factory.mktemp("exporter")
    for f in INPUTS:
        shutil.copy(os.path.join(SHIPPED, f), d / f)
    subprocess.run([exe, "-D0.850", "-E3.975", "-d6.500", "-T0.615", "-c0.0050", "-f0.050", "-s1"], cwd=d, check=True,
                   capture_output=True)
    return d


def test_exporter_files_equal_reference_exporter(reference_outputs, tmp_path):
    d = reference_outputs
    s = System.load(*(str(d / f) for f in INPUTS), T=0.615, box=350.0, c_mg=0.005, c_k=0.05, seed=1, rng=0)
    s.write_ninfo(str(tmp_path / "a.ninfo"))
    s.write_psf(str(tmp_path / "a.psf"))
    s.write_cgpdb(str(tmp_path / "a.cg.pdb"))
    for ours, theirs in (("a.ninfo", "16SCD_ninfo.ninfo"), ("a.psf", "16SCD_ninfo.psf"),
                         ("a.cg.pdb", "16SCD_ninfo.cg.pdb")):
        a = (tmp_path / ours).read_bytes()
        b = (d / theirs).read_bytes()
        assert len(b) > 1000 and a == b, theirs


def test_ninfo_records_of_the_small_system(tmp_path):
    s = load(golden_inputs(), "small")
    sd = s.to_dict()
    path = str(tmp_path / "small.ninfo")
    s.write_ninfo(path)
    kinds = [ln.split()[0] for ln in open(path)]
    count = {k: kinds.count(k) for k in set(kinds)}
    n_st3, n_st2, n_hb = len(sd["st3_E"]), len(sd["st2_E"]), len(sd["hb_E"])
    nbond = int(np.sum(sd["bt_kind"] == 0))
    nangl = int(np.sum(sd["bt_kind"] == 1))
    assert count["bond"] == nbond and count["angl"] == nangl
    assert count["tbs-dist"] == n_st3 and count["tbs-angl"] == 2 * n_st3 and count["tbs-dihd"] == 3 * n_st3
    assert count["bs-dist"] == n_st2 and count["bs-dihd"] == 2 * n_st2
    assert count["hb-dist"] == n_hb and count["hb-angl"] == 2 * n_hb and count["hb-dihd"] == 3 * n_hb
    # the records come in the exporter's order: bonded, stacks, H-bonds
    order = ["bond", "angl", "tbs-dist", "tbs-angl", "tbs-dihd", "bs-dist", "bs-dihd", "hb-dist", "hb-angl", "hb-dihd"]
    first = {k: kinds.index(k) for k in order if k in count}
    assert first["tbs-dist"] > max(first["bond"], first["angl"]) and first["hb-dist"] > first["bs-dist"]
