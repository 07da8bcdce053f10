"""The allocation-free list build (tis_pair_lists_noalloc) against the engine's own
list build (tis_populate_lists + tis_get_pairs) on the same coordinates.

Some callers cannot allocate device memory when they need a neighbour list: a
host recording its work into a CUDA graph (cudaMalloc cannot be captured), a time
step that must not synchronise the device (cudaFree does), an engine with a fixed,
pre-reserved memory budget.  The entry point keeps its scratch in a fixed device
array shared by every call, so two calls in a row on different systems also
check that nothing of the first call leaks into the second.  Pair sets are
integer data: they must be identical.  This file sorts last so that a run which
stops at the first failure has already run every other test."""
import numpy as np
import pytest

from systems import golden_inputs, load, pair_set
from tis_gb300 import Engine, api

pytestmark = pytest.mark.gpu


def _reference_lists(s):
    e = Engine([s], full_lists=1)  # the reference's full SR set, as the no-alloc build returns
    e.populate_lists()
    return e.pairs(0, 0), e.pairs(0, 1)


def _noalloc_lists(s):
    import torch
    d = s.to_dict()
    n = int(d["n_particles"][0])
    dev = torch.device("cuda:0")
    x, y, z = (torch.from_numpy(d[k]).to(dev) for k in ("x", "y", "z"))
    kind = torch.from_numpy(d["kind"].astype(np.int32)).to(dev)
    cap = 400 * n
    sr = torch.full((2 * cap,), -1, dtype=torch.int32, device=dev)
    lr = torch.full((2 * cap,), -1, dtype=torch.int32, device=dev)
    counts = torch.zeros(3, dtype=torch.int64, device=dev)
    stream = torch.cuda.current_stream().cuda_stream
    api.pair_lists_noalloc(x.data_ptr(), y.data_ptr(), z.data_ptr(), kind.data_ptr(), n, d["box"], 12.0 + 3.0,
                           float(d["rc"][0]) + 3.0, sr.data_ptr(), cap, lr.data_ptr(), cap, counts.data_ptr(),
                           stream)
    torch.cuda.synchronize()
    c = counts.cpu().numpy()
    assert c[0] <= cap and c[1] <= cap and c[2] == 0, c
    return (pair_set(sr[: 2 * c[0]].cpu().numpy()), pair_set(lr[: 2 * c[1]].cpu().numpy()))


def test_noalloc_lists_match_engine_lists_two_calls(synth_dir):
    systems = [load(synth_dir["central"], "central"), load(golden_inputs(), "small")]
    for s in systems:  # two calls in a row, different sizes, one shared scratch array
        want_sr, want_lr = _reference_lists(s)
        got_sr, got_lr = _noalloc_lists(s)
        assert len(want_sr) > 0 and len(want_lr) > 0
        assert np.array_equal(got_sr, want_sr)
        assert np.array_equal(got_lr, want_lr)


def test_noalloc_rejects_sizes_beyond_its_limit():
    big = np.zeros(1)
    with pytest.raises(api.TisError) as e:
        api.pair_lists_noalloc(1, 1, 1, 1, 70000, np.array([350.0] * 3), 15.0, 33.0, 1, 1, 1, 1, 1, None)
    assert e.value.code == 1 and "65536" in str(e.value)
    del big
