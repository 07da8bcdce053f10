"""Step graphs replaced while earlier graphs of the handle may still run: a handle
of several replica groups stepped by counts whose remainders change from call to
call, with no synchronisation between the calls, so that the remainder graph is
captured, instantiated and uploaded again right after the full graph was launched,
and handles created and destroyed in a row as the autotuner does.  The states equal
those of direct launches bit for bit (mixed precision: fixed-point sums)."""
import numpy as np
import pytest

from systems import golden_inputs, load
from tis_gb300 import PREC_MIXED, STATE_NAMES, Engine

pytestmark = pytest.mark.gpu

COUNTS = [57, 23, 110, 7, 63, 150, 41, 99]


@pytest.fixture(scope="module")
def replicas():
    return [load(golden_inputs(), "small", seed=s) for s in (3, 4, 5, 6, 7, 8)]


def _states(systems, **kw):
    e = Engine(systems, precision=PREC_MIXED, groups=3, **kw)
    e.populate_lists()
    for n in COUNTS:
        e.step(n)
    e.sync()
    st = e.get_states()
    e.close()
    return st


def test_remainder_graphs_recaptured_while_running(replicas):
    ref = _states(replicas, use_graph=0)
    for _ in range(3):  # handles created and destroyed in a row
        got = _states(replicas, use_graph=1, graph_steps=50)
        for k in STATE_NAMES:
            assert np.array_equal(got[k], ref[k]), k
