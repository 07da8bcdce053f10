"""The C-ABI library loads on a machine without a GPU and exports every entry
point include/tis_gpu.h declares.  No compute calls."""
import ctypes as C
import os
import re

import numpy as np
import pytest

from conftest import HAS_GPU, ROOT
from oracle_bridge import ensure_oracle
from tis_gb300 import api


def _declared():
    text = open(os.path.join(ROOT, "include", "tis_gpu.h")).read()
    return sorted(set(re.findall(r"^int\s+(tis_\w+)\s*\(", text, flags=re.M)))


def test_header_symbols_exported():
    lib = api.lib()
    names = _declared()
    assert len(names) >= 30
    for n in names:
        assert hasattr(lib, n), n
    assert sorted(api.EXPORTED) == names


def test_rand_stream_matches_oracle_stream():
    """The GPU path's rand() replacement and the oracle's are the same stream."""
    olib = C.CDLL(ensure_oracle())
    olib.tis_o_philox_word.restype = C.c_uint32
    olib.tis_o_philox_word.argtypes = [C.c_uint32] * 6 + [C.c_int]
    seed = 0x1234567890ABCDEF
    got = api.rand_stream(seed, 1000, 64)
    want = []
    for k in range(1000, 1064):
        w = olib.tis_o_philox_word((k >> 2) & 0xffffffff, k >> 34, 0, 0, seed & 0xffffffff, seed >> 32, k & 3) >> 1
        want.append(w if w else 1)
    assert list(got) == want


def test_default_run_params_follow_reference():
    p = api.run_params()
    assert (p.sr, p.skin, p.lr_interval) == (12.0, 3.0, 10)  # E:6227-6229, E:2550


@pytest.mark.skipif(HAS_GPU, reason="checks the no-GPU error path")
def test_create_without_gpu_fails_cleanly():
    from systems import golden_inputs, load
    s = load(golden_inputs(), "small")
    with pytest.raises(api.TisError) as e:
        api.Engine([s])
    assert e.value.code == 4
