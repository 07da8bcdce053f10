"""The reference's output files (Contacts / Coordinates / Energies, E:6276-6312),
its restart read (E:6181-6211) and the tis_run command line."""
import os
import shutil
import subprocess

import numpy as np
import pytest

from systems import golden_inputs, load
from tis_gb300 import Engine, read_last_frame, TisError
from tis_gb300 import build as _build


def _write_frames(path, frames):
    """Frames in the reference's Coordinates layout: x, y, z as 1-based arrays (n+1 doubles)."""
    with open(path, "wb") as f:
        for x, y, z in frames:
            for a in (x, y, z):
                np.concatenate([[0.0], a]).astype(np.float64).tofile(f)


def test_read_last_frame(tmp_path):
    n = 7
    rng = np.random.default_rng(3)
    frames = [tuple(rng.normal(size=n) for _ in range(3)) for _ in range(3)]
    p = str(tmp_path / "coords.dat")
    _write_frames(p, frames)
    x, y, z, count = read_last_frame(p, n)
    assert count == 3
    assert np.array_equal(x, frames[-1][0]) and np.array_equal(y, frames[-1][1]) and np.array_equal(z, frames[-1][2])
    with open(p, "ab") as f:
        f.write(b"\0" * 16)
    with pytest.raises(TisError) as err:
        read_last_frame(p, n)
    assert err.value.code == 3


@pytest.mark.gpu
def test_write_frame_matches_the_engine(tmp_path):
    s = load(golden_inputs(), "small")
    e = Engine([s])
    e.populate_lists()
    e.step(60)
    e.sync()
    paths = [str(tmp_path / k) for k in ("contacts.dat", "coordinates.dat", "energies.dat")]
    for _ in range(2):
        e.write_frame(0, *paths)
    st = e.get_state(0)
    en = e.energies(0)
    stacks = e.stack_energies(0)
    lines = open(paths[0]).read().splitlines()
    assert len(lines) == 2
    vals = lines[0].split()
    assert len(vals) == len(stacks)
    assert vals == [f"{v:+.3f}" for v in stacks]
    x, y, z, count = read_last_frame(paths[1], e.n[0])
    assert count == 2
    assert np.array_equal(x, st["x"]) and np.array_equal(y, st["y"]) and np.array_equal(z, st["z"])
    row = [float(v) for v in open(paths[2]).read().splitlines()[0].split()]
    want = [en[0], en[1], en[2], float(np.sum(stacks)), en[4]]
    np.testing.assert_allclose(row, want, rtol=1e-6, atol=1e-6)


@pytest.mark.gpu
def test_cli_runs_writes_and_restarts(tmp_path):
    _build.build()
    g = golden_inputs()
    for src, dst in [(g["pdb"], "16SCD.pdb"), (g["bonds"], "16SCD_16SCD_unprocessed_bonds.dat"),
                     (g["stacks"], "16SCD_16SCD_unprocessed_stacks.dat"), (g["maxikey"], "MAXIKEY_Mg_Cl_K.dat")]:
        shutil.copy(src, tmp_path / dst)
    args = [_build.RUN, "-T0.59219", "-c0.005", "-f0.05", "-s3", "--box", "200", "--rc", "30", "--center", "100",
            "--every", "50", "--snapshot-every", "100", "--replicas", "2"]
    subprocess.run(args + ["--steps", "200"], cwd=tmp_path, check=True, capture_output=True, text=True, timeout=300)
    tail = "D0.850_E3.975_d6.500_T0.592_cM0.0050_f0.050_s{}"
    for seed in (3, 4):
        base = tail.format(seed)
        energies = (tmp_path / f"Energies_16SCD_EPS_Mg_Cl_K_{base}.dat").read_text().splitlines()
        assert len(energies) == 4  # steps 50, 100, 150, 200
        assert all(len(l.split()) == 5 for l in energies)
        assert (tmp_path / f"Contacts_16SCD_EPS_Mg_Cl_K_{base}_2.dat").exists()  # snapshot at step 200
        coords = tmp_path / f"Coordinates_16SCD_EPS_Mg_Cl_K_{base}.dat"
        assert coords.stat().st_size % (3 * 8) == 0
    subprocess.run(args + ["--steps", "400"], cwd=tmp_path, check=True, capture_output=True, text=True, timeout=300)
    base = tail.format(3)
    energies = (tmp_path / f"Energies_16SCD_EPS_Mg_Cl_K_{base}.dat").read_text().splitlines()
    assert len(energies) == 8  # resumed at step 4 x 50 from the last frame, then frames at 250 .. 400


@pytest.mark.gpu
@pytest.mark.parametrize("kind,radius", [(3, 4.4), (3, 7.2684), (5, 5.0), (5, 7.2684), (4, 7.2684), (0, 7.3)])
def test_ion_counts_match_a_direct_count(kind, radius):
    """Ions of one kind within a radius of each phosphate (the reference's bound-ion
    analyses), counted on the device from the SR lists, equal a direct count over
    all ions with the engine's image rule."""
    s = load(golden_inputs(), "small")
    e = Engine([s])
    e.populate_lists()
    e.step(150)
    e.sync()
    counts, total = e.ion_counts(0, kind, radius)
    st = e.get_state(0)
    sd = s.to_dict()
    kinds = np.asarray(sd["kind"])
    L = np.asarray(sd["box"], dtype=np.float64)
    X = np.stack([st["x"], st["y"], st["z"]], 1)
    P = np.nonzero(kinds == 0)[0]
    ions = np.nonzero(kinds == kind)[0]
    d = X[P][:, None, :] - X[ions][None, :, :]
    d = np.where(d > 0.5 * L, d - L, d)
    d = np.where(d < -0.5 * L, d + L, d)
    r2 = (d[..., 0] * d[..., 0] + d[..., 1] * d[..., 1]) + d[..., 2] * d[..., 2]
    if kind == 0:  # phosphates around phosphates: not itself
        r2[np.arange(len(P)), np.arange(len(P))] = np.inf
    within = r2 <= radius * radius
    assert np.array_equal(counts, within.sum(1))
    assert total == int(within.any(0).sum())


def test_psf_matches_the_exporter_layout(tmp_path):
    """tis_write_psf: the layout of the reference's topology exporter
    (analysis/make_ninfo/16SCD_ninfo.cpp:6563-6650): atom records with residue
    names R<base>, atom names S / <base>b / P and ions, charges, the chain bonds."""
    s = load(golden_inputs(), "small")
    p = str(tmp_path / "t.psf")
    s.write_psf(p)
    lines = open(p).read().split("\n")
    n, ntp = int(s["n_particles"][0]), int(s["n_rna"][0])
    assert lines[0] == f"{n:8d} !NATOM"
    atoms = lines[1:1 + n]
    letter = {3: "A", 4: "G", 5: "C", 6: "U"}
    typ, kind = s["type"], s["kind"]
    for i in range(1, ntp + 1):
        a = atoms[i - 1]
        c = letter[typ[3 * (i // 3) + 1]]
        assert int(a[:8]) == i and a[8:11] == f"R{c} " and int(a[11:15]) == i // 3 + 1
        assert a[15:23] == f"      R{c}"
        name = a[23:29].strip()
        assert name == ("S" if i % 3 == 1 else f"{c}b" if i % 3 == 2 else "P")
        assert float(a[37:48]) == (-1.0 if i % 3 == 0 else 0.0) and float(a[48:62]) == 10.0
        assert a.endswith("           0")
    charges = {3: 2.0, 4: -1.0, 5: 1.0}
    for i in range(ntp + 1, n + 1):
        a = atoms[i - 1]
        assert float(a[37:48]) == charges[kind[i - 1]]
        assert int(a[11:15]) == ntp // 3 + i - ntp + 1
    assert lines[1 + n] == f"{ntp - 1:8d} !NBOND"
    ints = [int(t) for ln in lines[2 + n:] for t in [ln[k:k + 8] for k in range(0, len(ln), 8)] if t.strip()]
    pairs = list(zip(ints[0::2], ints[1::2]))
    assert len(pairs) == ntp - 1
    assert pairs[0] == (1, 2) and pairs[1] == (1, 3) and pairs[2] == (3, 4) and pairs[3] == (4, 5)


def _read_dcd(path):
    """Frames of a CHARMM/NAMD DCD file: (n_set, natom, [frames of (3, natom) float32])."""
    raw = open(path, "rb").read()
    i32 = lambda o: int(np.frombuffer(raw, np.int32, 1, o)[0])
    assert i32(0) == 84 and raw[4:8] == b"CORD" and i32(88) == 84
    nset, nsavc = i32(8), i32(16)
    o = 92
    tlen = i32(o)
    o += 4 + tlen + 4
    assert i32(o) == 4
    natom = i32(o + 4)
    o += 12
    frames = []
    while o < len(raw):
        xyz = []
        for _ in range(3):
            assert i32(o) == 4 * natom
            xyz.append(np.frombuffer(raw, np.float32, natom, o + 4))
            o += 4 * natom + 8
        frames.append(np.stack(xyz))
    return nset, nsavc, natom, frames


@pytest.mark.gpu
def test_dcd_frames_equal_the_engine_positions(tmp_path):
    s = load(golden_inputs(), "small")
    e = Engine([s])
    e.populate_lists()
    p = str(tmp_path / "t.dcd")
    want = []
    for _ in range(3):
        e.step(10)
        e.write_dcd(0, p, 10)
        st = e.get_state(0)
        want.append(np.stack([st["x"], st["y"], st["z"]]).astype(np.float32))
    nset, nsavc, natom, frames = _read_dcd(p)
    assert (nset, nsavc, natom) == (3, 10, e.n[0]) and len(frames) == 3
    for a, b in zip(frames, want):
        assert np.array_equal(a, b)
    e.close()


def test_cgpdb_matches_the_exporter_layout(tmp_path):
    """tis_write_cgpdb: the exporter's RECORD counts, bead and ion records in PDB
    columns (16SCD_ninfo.cpp:6479-6561), coordinates to 1e-3 A."""
    s = load(golden_inputs(), "small")
    p = str(tmp_path / "t.pdb")
    s.write_cgpdb(p)
    lines = open(p).read().splitlines()
    n, ntp, nbp = int(s["n_particles"][0]), int(s["n_rna"][0]), int(s["n_entries"][0])
    want = [("N_amino", nbp), ("NBP_atom", nbp), ("NB_atom", nbp + n - ntp), ("NTP_atom", ntp),
            ("NpTP_atom", ntp * (ntp + 1) // 2), ("NT_atom", n)]
    for ln, (k, v) in zip(lines[:6], want):
        assert ln.split() == ["RECORD", k, str(v)]
    atoms = lines[6:6 + ntp]
    assert lines[6 + ntp] == "TER" and lines[-1] == "TER" and len(lines) == 6 + n + 2
    x, y, z = s["x"], s["y"], s["z"]
    letter = {3: "A", 4: "G", 5: "C", 6: "U"}
    for i, a in enumerate(atoms, start=1):
        c = letter[s["type"][3 * (i // 3) + 1]]
        assert a[:6] == "ATOM  " and int(a[6:11]) == i
        assert a[12:16] == (" S  " if i % 3 == 1 else f" {c}b " if i % 3 == 2 else " P  ")
        assert a[17:20] == f"R{c} " [:3] and a[21] == "A" and int(a[22:26]) == i // 3 + 1
        assert [float(a[30:38]), float(a[38:46]), float(a[46:54])] == pytest.approx([x[i - 1], y[i - 1], z[i - 1]], abs=6e-4)
    names = {3: "MG    MG", 4: " Cl   Cl", 5: " K    K "}
    for i in range(ntp + 1, n + 1):
        a = lines[6 + i]
        assert int(a[6:11]) == i and a[12:20] == names[s["kind"][i - 1]] and a[21] == "B" and int(a[22:26]) == i


def test_contact_concentration_formula():
    """integrate_num_ions.py:51-55: count / (nstep 4/3 pi cut^3 6.02214 / 10^4) mol/L."""
    import math
    from tis_gb300 import contact_concentration
    cut = 7.300000001
    got = contact_concentration([12, 0, 3], 40)
    want = [c / (40 * 4 / 3.0 * math.pi * (cut ** 3) * 6.02214 / (10 ** 4)) for c in (12, 0, 3)]
    assert np.allclose(got, want, rtol=1e-15)


@pytest.mark.gpu
def test_checkpoint_resumes_bit_for_bit(tmp_path):
    """tis_checkpoint_save / _load: a fresh handle continues exactly as the saving
    one (lists, held LR force, counters and rand() positions included)."""
    systems = [load(golden_inputs(), "small", seed=s) for s in (3, 4, 5)]
    path = str(tmp_path / "run.ckpt")
    a = Engine(systems, groups=2)
    a.populate_lists()
    a.step(137)  # mid-interval of the LR refresh, lists some steps old
    a.checkpoint_save(path)
    a.step(150)
    ref = a.get_states()
    ref_c = [a.counters(r) for r in range(3)]
    b = Engine(systems, groups=2)
    b.checkpoint_load(path)
    b.step(150)
    got = b.get_states()
    for k in ref:
        assert np.array_equal(got[k], ref[k]), k
    assert [b.counters(r) for r in range(3)] == ref_c
    c = Engine(systems, groups=1)
    with pytest.raises(TisError):
        c.checkpoint_load(path)


@pytest.mark.gpu
def test_checkpoint_load_refuses_other_systems_and_damaged_files(tmp_path):
    """A checkpoint loads only onto a handle of the same systems, parameters and
    seeds; a truncated file or one with trailing bytes is refused; a refused load
    leaves the handle's state untouched."""
    systems = [load(golden_inputs(), "small", seed=s) for s in (3, 4)]
    path = str(tmp_path / "run.ckpt")
    a = Engine(systems)
    a.populate_lists()
    a.step(60)
    a.checkpoint_save(path)
    data = open(path, "rb").read()
    other = Engine([load(golden_inputs(), "small", seed=s) for s in (3, 5)])  # same sizes, another seed
    other.populate_lists()
    other.step(10)
    before = other.get_states()
    cases = {"seed": path}
    for name, blob in (("truncated", data[:-1000]), ("trailing", data + b"x")):
        cases[name] = str(tmp_path / f"{name}.ckpt")
        open(cases[name], "wb").write(blob)
    for name, p in cases.items():
        with pytest.raises(TisError) as err:
            other.checkpoint_load(p)
        assert err.value.code == 3, name  # TIS_ERR_FORMAT
        after = other.get_states()
        for k in before:
            assert np.array_equal(after[k], before[k]), (name, k)
    b = Engine(systems)
    b.checkpoint_load(cases["seed"])  # the saving handle's systems accept it


@pytest.mark.gpu
def test_cli_checkpoint_continues_bit_for_bit(tmp_path):
    """tis_run --checkpoint: a run stopped at step 200 and started again to 400
    writes the same files, frame for frame, as one run to 400; --dcd appends every
    frame to a trajectory."""
    _build.build()
    g = golden_inputs()
    args = [_build.RUN, "-T0.59219", "-c0.005", "-f0.05", "-s3", "--box", "200", "--rc", "30", "--center", "100",
            "--every", "50", "--snapshot-every", "0", "--replicas", "2", "--checkpoint", "run.ckpt", "--dcd"]
    for d in ("split", "whole"):
        (tmp_path / d).mkdir()
        for src, dst in [(g["pdb"], "16SCD.pdb"), (g["bonds"], "16SCD_16SCD_unprocessed_bonds.dat"),
                         (g["stacks"], "16SCD_16SCD_unprocessed_stacks.dat"), (g["maxikey"], "MAXIKEY_Mg_Cl_K.dat")]:
            shutil.copy(src, tmp_path / d / dst)
    for steps in ("200", "400"):
        subprocess.run(args + ["--steps", steps], cwd=tmp_path / "split", check=True, capture_output=True, text=True,
                       timeout=300)
    subprocess.run(args + ["--steps", "400"], cwd=tmp_path / "whole", check=True, capture_output=True, text=True,
                   timeout=300)
    base = "16SCD_EPS_Mg_Cl_K_D0.850_E3.975_d6.500_T0.592_cM0.0050_f0.050_s{}"
    for seed in (3, 4):
        for kind, ext in (("Coordinates", "dat"), ("Energies", "dat"), ("Contacts", "dat"), ("Trajectory", "dcd")):
            name = f"{kind}_{base.format(seed)}.{ext}"
            a = (tmp_path / "split" / name).read_bytes()
            b = (tmp_path / "whole" / name).read_bytes()
            assert a == b, name
        energies = (tmp_path / "whole" / f"Energies_{base.format(seed)}.dat").read_text().splitlines()
        assert len(energies) == 8
        nset, _, _, frames = _read_dcd(str(tmp_path / "whole" / f"Trajectory_{base.format(seed)}.dcd"))
        assert nset == 8 and len(frames) == 8


def test_cli_without_inputs_or_gpu_fails_cleanly(tmp_path):
    """tis_run reports a missing input file (or, on a machine without a GPU, the
    missing device) as an error message and exit status 1, without a crash."""
    _build.build()
    r = subprocess.run([_build.RUN, "--steps", "10"], cwd=tmp_path, capture_output=True, text=True, timeout=120)
    assert r.returncode == 1
    assert "tis_run:" in r.stderr and "error" in r.stderr


@pytest.mark.gpu
@pytest.mark.parametrize("fused", [0, 2])
def test_frames_written_from_inside_the_step(synth_dir, fused):
    """tis_frames_*: the frames the step's kernels write into the host ring equal
    the states and Energies-file values of the same run stopped at those steps
    (Rg within rounding: its block sum runs over other threads); an overwritten,
    an unreached and a non-frame step are refused; the ring changes no result."""
    specs = [dict(seed=3 + 2 * k, n_mg=10 + 4 * k, n_cl=261 + 8 * k, n_k=317) for k in range(3)]
    systems = [load(synth_dir["small"], "small", **sp) for sp in specs]
    kw = dict(groups=2, graph_steps=40, fused_ctas=fused)
    a = Engine(systems, **kw)
    ring = a.frames_start(20, depth=3)
    a.populate_lists()
    a.step(100)  # frames at steps 20, 40, ..., 100; the ring keeps 60, 80, 100
    frames = {k: ring.read(k) for k in (100, 80, 60)}
    for bad in (40, 120, 30):  # overwritten, not reached, not a frame step
        with pytest.raises(TisError):
            ring.read(bad)
    b = Engine(systems, **kw)
    b.populate_lists()
    done = 0
    for k in (60, 80, 100):
        b.step(k - done)
        done = k
        st = b.get_states(("x", "y", "z"))
        en = b.all_energies()
        for c in ("x", "y", "z"):
            assert np.array_equal(frames[k][c], st[c]), (k, c)
        assert np.array_equal(frames[k]["energies"][:, :4], en[:, :4]), k
        np.testing.assert_allclose(frames[k]["energies"][:, 4], en[:, 4], rtol=1e-12)
    fa, fb = a.get_states(), b.get_states()
    for k in fa:
        assert np.array_equal(fa[k], fb[k]), k
    ring.stop()
    a.step(20)  # detached: stepping goes on without a ring
    a.sync()
