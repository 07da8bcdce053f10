"""Device ion density grids (tis_density_*) against numpy.histogramdd of the same
frames (the reference's analysis/Mg_distribution_3D/calc_Mg_density.py bins with
it), with and without the least-squares fit of a bead selection (its
bestfit_motifs.py); the OpenDX file read back the way search_dx_maxvalue.py reads
it."""
import numpy as np
import pytest

from systems import golden_inputs, load
from tis_gb300 import PREC_MIXED, Engine

pytestmark = pytest.mark.gpu

K_ION = 5  # part_key of K+


def _kabsch(x, y):
    """Rotation R and centroids with y ~ R (x - xc) + yc (least squares, proper rotation)."""
    xc, yc = x.mean(0), y.mean(0)
    H = (x - xc).T @ (y - yc)
    U, _, Vt = np.linalg.svd(H)
    d = np.sign(np.linalg.det(Vt.T @ U.T))
    return Vt.T @ np.diag([1.0, 1.0, d]) @ U.T, xc, yc


def _frames(engine, grid, n, kinds, fit=None):
    """n frames 20 steps apart, each added to the grid; returns the ions' positions
    (moved by the numpy fit when fit = (beads, ref)) and the fits' rmsds."""
    pts, rmsd = [], []
    for _ in range(n):
        engine.step(20)
        grid.add()
        st = engine.get_state(0)  # synchronises: the frame the grid binned
        xyz = np.stack([st["x"], st["y"], st["z"]], 1)
        ions = xyz[kinds == K_ION]
        if fit is not None:
            beads, ref = fit
            R, xc, yc = _kabsch(xyz[beads], ref)
            ions = (ions - xc) @ R.T + yc
            moved = (xyz[beads] - xc) @ R.T + yc
            rmsd.append(np.sqrt(((moved - ref) ** 2).sum(1).mean()))
        pts.append(ions)
    return pts, rmsd


def _hist(pts, lo, delta, dims):
    edges = [lo[a] + delta * np.arange(dims[a] + 1) for a in range(3)]
    return sum(np.histogramdd(p, bins=edges)[0] for p in pts), edges


def test_density_matches_histogramdd(tmp_path):
    s = load(golden_inputs(), "small")
    kinds = s["kind"]
    e = Engine([s], precision=PREC_MIXED)
    e.populate_lists()
    lo, delta, dims = (0.0, 0.0, 0.0), 5.0, (40, 40, 40)  # the 200 A box
    g = e.density(0, K_ION, lo, delta, dims)
    pts, _ = _frames(e, g, 6, kinds)
    counts, frames, _ = g.get()
    want, _ = _hist(pts, lo, delta, dims)
    assert frames == 6
    assert counts.sum() == 6 * np.count_nonzero(kinds == K_ION)
    assert np.array_equal(counts, want)

    # the OpenDX file, parsed as search_dx_maxvalue.py parses it
    path = str(tmp_path / "k.dx")
    g.write_dx(path)
    lines = open(path).read().splitlines()
    assert lines[6].split()[-3:] == ["40", "40", "40"]
    assert [float(v) for v in lines[7].split()[1:]] == [2.5, 2.5, 2.5]
    tok = lines[12].split()
    n = int(tok[9])
    assert n == counts.size
    vals = []
    for ln in lines[13:13 + (n + 2) // 3]:
        vals += [float(v) for v in ln.split()]
    assert np.array_equal(np.array(vals), counts.ravel())
    g.close()
    e.close()


def test_density_fit_matches_least_squares_superposition():
    s = load(golden_inputs(), "small")
    kinds = s["kind"]
    e = Engine([s], precision=PREC_MIXED)
    e.populate_lists()
    st0 = e.get_state(0)
    beads = np.arange(0, 60, 2)
    x0 = np.stack([st0["x"], st0["y"], st0["z"]], 1)[beads]
    a = 0.7
    rot = np.array([[np.cos(a), -np.sin(a), 0.0], [np.sin(a), np.cos(a), 0.0], [0.0, 0.0, 1.0]])
    ref = x0 @ rot.T + np.array([13.0, -7.0, 2.5])  # the motif moved: the fit must undo it
    lo, delta, dims = (-400.0, -400.0, -400.0), 10.0, (100, 100, 100)
    g = e.density(0, K_ION, lo, delta, dims, fit_beads=beads, fit_ref=ref)
    pts, rmsds = _frames(e, g, 5, kinds, fit=(beads, ref))
    counts, frames, rmsd = g.get()
    want, edges = _hist(pts, lo, delta, dims)
    assert counts.sum() == want.sum() == 5 * np.count_nonzero(kinds == K_ION)
    near = sum(int((np.abs((p[:, a:a + 1] - edges[a][None, :])) < 1e-7).sum()) for p in pts for a in range(3))
    assert np.abs(counts - want).sum() <= 2 * near
    assert rmsd == pytest.approx(rmsds[-1], rel=1e-9, abs=1e-12)
    g.close()
    e.close()


def test_density_rejects_bad_grids():
    from tis_gb300 import TisError
    s = load(golden_inputs(), "small")
    e = Engine([s], precision=PREC_MIXED)
    with pytest.raises(TisError):
        e.density(0, K_ION, (0, 0, 0), 0.0, (10, 10, 10))
    with pytest.raises(TisError):
        e.density(0, K_ION, (0, 0, 0), 1.0, (10, 0, 10))
    with pytest.raises(TisError):
        e.density(0, K_ION, (0, 0, 0), 1.0, (10, 10, 10), fit_beads=[0, 1], fit_ref=np.zeros((2, 3)))
    e.close()


def test_density_outliving_its_handle_reports_state_error():
    from tis_gb300 import TisError
    s = load(golden_inputs(), "small")
    e = Engine([s], precision=PREC_MIXED)
    e.populate_lists()
    g = e.density(0, K_ION, (0, 0, 0), 10.0, (20, 20, 20))
    g.add()
    e.close()  # releases the grid's device memory
    with pytest.raises(TisError) as err:
        g.get()
    assert err.value.code == 8
    g.close()
