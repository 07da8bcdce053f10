"""The integer forms of the reference's rand() arithmetic used by the kernels
(u31_ratio: (double) rand () / RAND_MAX; pick_index: ceil(u n) with the
reference's clamps, E:2245-2262) equal the FP64 expressions they replace.  The
host build of the same header functions is checked here on 2^24 + edge values
(u31_ratio was also checked on all 2^31 - 1 draws) and 10^7 random (v, n)."""
import os
import shutil
import subprocess
import tempfile

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
CSRC = os.path.join(ROOT, "16s-central-folding_gb300", "csrc")

PROGRAM = r"""
#include <cmath>
#include <cstdio>
#include <cstring>
#include "tis_device.cuh"
int main() {
    unsigned long long bad = 0, n_checked = 0;
    auto check_u = [&](uint32_t v) {
        double a = tis::u31_ratio(v), b = (double)v / 2147483647.0;
        bad += memcmp(&a, &b, 8) != 0;
        ++n_checked;
    };
    for (uint32_t v = 1; v < 2147483647u - 128u; v += 127u) check_u(v);
    for (uint32_t v = 1; v < 4096u; ++v) check_u(v);
    for (uint32_t v = 2147483647u - 4096u; v <= 2147483647u; ++v) check_u(v);
    for (int s = 0; s < 31; ++s) { check_u(1u << s); check_u((1u << s) + 1u); if (s) check_u((1u << s) - 1u); }
    unsigned long long bad_pick = 0;
    unsigned long long x = 88172645463325252ull;
    for (int it = 0; it < 10000000; ++it) {
        x ^= x << 13; x ^= x >> 7; x ^= x << 17;
        uint32_t v = (uint32_t)(x % 2147483647ull) + 1u;
        int n = (int)((x >> 40) % 4096) + 1;
        int j = (int)ceil((double)v / 2147483647.0 * n);
        if (j == n + 1) j = n;
        if (j == 0) j = 1;
        bad_pick += j != tis::pick_index(v, n);
    }
    printf("%llu %llu %llu\n", n_checked, bad, bad_pick);
    return 0;
}
"""


def test_integer_rand_arithmetic_matches_fp64():
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    with tempfile.TemporaryDirectory() as tmp:
        src = os.path.join(tmp, "t.cpp")
        exe = os.path.join(tmp, "t")
        with open(src, "w") as f:
            f.write(PROGRAM)
        subprocess.run([gxx, "-O2", "-std=c++17", "-ffp-contract=off", "-I", CSRC, "-I", "/usr/local/cuda/include",
                        src, "-o", exe], check=True, capture_output=True, text=True)
        out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    n_checked, bad, bad_pick = map(int, out)
    assert n_checked > 16_000_000
    assert bad == 0
    assert bad_pick == 0
