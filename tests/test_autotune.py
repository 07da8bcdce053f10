"""The launch-configuration autotuner (tis_autotune) and the launch shapes it
chooses between: in mixed precision every shape gives bit-identical states
(fixed-point sums), so the choice is by speed alone."""
import time

import numpy as np
import pytest

from systems import golden_inputs, load
from tis_gb300 import PREC_MIXED, STATE_NAMES, Engine, TisError, autotune

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def replicas():
    return [load(golden_inputs(), "small", seed=s) for s in (3, 4, 5, 6)]


def _run(systems, steps, **kw):
    e = Engine(systems, precision=PREC_MIXED, **kw)
    e.populate_lists()
    e.step(steps)
    e.sync()
    st = e.get_states()
    e.close()
    return st


@pytest.mark.parametrize("lanes_sr,lanes_lr", [(2, 8), (4, 2), (1, 4)])
def test_launch_shapes_give_identical_states(replicas, lanes_sr, lanes_lr):
    ref = _run(replicas, 150)
    got = _run(replicas, 150, lanes_sr=lanes_sr, lanes_lr=lanes_lr, groups=2, graph_steps=25)
    for k in STATE_NAMES:
        assert np.array_equal(got[k], ref[k]), k


def test_bad_launch_shape_is_rejected(replicas):
    with pytest.raises(TisError):
        Engine(replicas, lanes_sr=3)
    with pytest.raises(TisError):
        Engine(replicas, lanes_lr=16)


def test_autotune_chooses_and_caches(replicas, tmp_path):
    cache = str(tmp_path / "tune.txt")
    best, rate = autotune(replicas, steps=100, cache=cache)
    assert 1 <= best["groups"] <= len(replicas)
    assert best["graph_steps"] in (25, 50, 100, 200)
    assert best["lanes_sr"] in (1, 2, 4) and best["lanes_lr"] in (2, 4, 8)
    assert best["fused_ctas"] in (0, 1, 2, 4)
    assert rate > 0
    with open(cache) as f:
        assert len(f.read().splitlines()) == 1
    t0 = time.perf_counter()
    again, rate2 = autotune(replicas, steps=100, cache=cache)
    assert time.perf_counter() - t0 < 5.0  # read from the cache, no trials
    assert again == best and rate2 == pytest.approx(rate, rel=1e-3)
    ref = _run(replicas, 60)  # the chosen configuration gives the default's states
    got = _run(replicas, 60, **best)
    for k in STATE_NAMES:
        assert np.array_equal(got[k], ref[k]), k
