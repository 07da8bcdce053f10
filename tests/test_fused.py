"""The persistent fused step kernel (tis_run_params.fused_ctas > 0): one
thread-block cluster per replica runs whole steps back to back.

In mixed precision it gives the chain of separate kernels' results bit for bit
(fixed-point force sums; the same per-item code): states, step, rebuild and
rand() counters, for any cluster size, with and without graph capture, on
replicas of different sizes and on the batched workload's own replicas.  In FP64
it tracks the oracle step for step like the separate kernels do."""
import numpy as np
import pytest

from oracle_bridge import Oracle
from systems import golden_inputs, load
from tis_gb300 import NOISE_REFERENCE, PREC_FP64, PREC_MIXED, Engine

pytestmark = pytest.mark.gpu


def _run(systems, steps, **kw):
    e = Engine(systems, **kw)
    e.populate_lists()
    e.step(steps)
    e.sync()
    out = [e.get_state(r) for r in range(len(systems))], [e.counters(r) for r in range(len(systems))]
    e.close()
    return out


def _same(a, b, label):
    for r, (sa, sb) in enumerate(zip(a[0], b[0])):
        for k in sa:
            assert np.array_equal(sa[k], sb[k]), (label, r, k)
    assert a[1] == b[1], (label, a[1], b[1])


def test_fused_equals_separate_kernels_bitwise(synth_dir):
    f = synth_dir["small"]
    specs = [dict(seed=3 + 2 * k, n_mg=10 + 3 * k, n_cl=261 + 6 * k, n_k=317) for k in range(5)]
    systems = [load(f, "small", **sp) for sp in specs]
    ref = _run(systems, 300, groups=2, graph_steps=50)
    assert all(c[1] > 1 for c in ref[1])  # list rebuilds happened inside the run
    for ctas in (1, 2, 4):
        for use_graph in (0, 1):
            got = _run(systems, 300, groups=2, graph_steps=50, fused_ctas=ctas, use_graph=use_graph)
            _same(ref, got, f"ctas {ctas} graph {use_graph}")


def test_fused_bench_replicas_bitwise():
    import tempfile

    import bench
    files = bench.make_inputs(tempfile.mkdtemp())
    specs = bench.replica_specs()
    systems = bench.load_systems(files, [specs[0], specs[31], specs[63]])
    ref = _run(systems, 400, graph_steps=100)
    got = _run(systems, 400, graph_steps=100, fused_ctas=2)
    _same(ref, got, "bench replicas")


def test_fused_fp64_tracks_oracle():
    s = load(golden_inputs(), "small")
    o = Oracle(s.to_dict(), seed=3)
    o.populate_lists()
    e = Engine([s], precision=PREC_FP64, noise=NOISE_REFERENCE, fused_ctas=2)
    e.populate_lists()
    o.step(200)
    e.step(200)
    e.sync()
    st, ost = e.get_state(0), o.get_state()
    d = max(np.abs(st[k] - ost[k]).max() for k in ("x", "y", "z"))
    assert d < 1e-7, d
    assert e.counters(0)[2] == o.draws()


def test_fused_launch_count(synth_dir):
    systems = [load(synth_dir["small"], "small", seed=s) for s in (3, 4)]
    e = Engine(systems, precision=PREC_MIXED, fused_ctas=2, use_graph=0, groups=1)
    e.populate_lists()
    n0 = e.launches()
    e.step(40)
    e.step(40)
    e.sync()
    assert e.launches() - n0 == 2  # one kernel per call and replica group
