#!/usr/bin/env python3
"""Build recipe for the reference engine as the CPU oracle (TEST INFRASTRUCTURE).

Makes a build-time copy of the reference's engine source under oracle/_ref/
(git-ignored), applies the patch table below, and compiles it together with
oracle/ref_harness.cpp into oracle/_ref/tis_ref.  Nothing of the reference is
committed to this repository.

Where the sources come from:
  1. $TIS_REFERENCE_ROOT/src/16SCD_Mg_Cl_K_COPY_fast.cpp, or /root/reference/src/...
  2. otherwise an existing oracle/_ref/engine_patched.cpp (a copy made earlier by
     this script on a machine that had the reference) is recompiled as it is.

Patch table (every item is a literal search/replace that must match exactly once;
E: = src/16SCD_Mg_Cl_K_COPY_fast.cpp):
  P1  E:10    after '#include <sys/timeb.h>' include tis_ref_hooks.h (hook
              declarations and the centre-atom variable).
  P2  E:2670  'adjust_box ( 500 );' -> 'adjust_box ( tis_center_atom );' so that
              systems with fewer than 500 RNA beads can be recentred (the literal
              500 reads past the end of x[] there).
  P3  E:925   first statement of bead_bond_force records the bond term (the hook
              is a no-op unless the harness is exporting the topology).
  P4  E:1032  first statement of bead_valence_force records the angle term.
Compile-time settings (not source edits):
  -Dmain=tis_ref_main        the harness owns main() and runs the set-up itself
  -include ref_rng_shim.h    rand()/srand() routed through the harness
  -I mpi_stub                single-rank MPI (no MPI library in these images)
  -ffp-contract=off          no FMA contraction on aarch64, so r^2 comparisons and
                             sums round exactly as the reference's x86 build did
The list capacities (E:6233-6235), box side (E:6076), Coulomb cutoff (E:348),
ion counts (E:6167-6171) and step count (E:6274) are globals or live in main();
the harness sets them at run time, so they need no source edit.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
REL = os.path.join("src", "16SCD_Mg_Cl_K_COPY_fast.cpp")

PATCHES = [
    ("P1", "#include <sys/timeb.h>\n", "#include <sys/timeb.h>\n#include \"tis_ref_hooks.h\"\n"),
    ("P2", "adjust_box ( 500 );", "adjust_box ( tis_center_atom );"),
    ("P3",
     "void bead_bond_force ( int i1, int i2, double k0, double r0 )\n{\n",
     "void bead_bond_force ( int i1, int i2, double k0, double r0 )\n{\n\ttis_hook_bond ( i1, i2, k0, r0 );\n"),
    ("P4",
     "void bead_valence_force ( int i1, int i2, int i3, double k0, double theta0 )\n{\n",
     "void bead_valence_force ( int i1, int i2, int i3, double k0, double theta0 )\n{\n"
     "\ttis_hook_angle ( i1, i2, i3, k0, theta0 );\n"),
]


def reference_source():
    roots = [os.environ.get("TIS_REFERENCE_ROOT"), "/root/reference"]
    for r in roots:
        if r and os.path.isfile(os.path.join(r, REL)):
            return os.path.join(r, REL)
    return None


def make_patched_copy(src):
    text = open(src, encoding="latin-1").read()
    for name, old, new in PATCHES:
        n = text.count(old)
        if n != 1:
            raise RuntimeError(f"patch {name}: anchor found {n} times (expected 1)")
        text = text.replace(old, new)
    os.makedirs(OUT, exist_ok=True)
    dst = os.path.join(OUT, "engine_patched.cpp")
    with open(dst, "w", encoding="latin-1") as f:
        f.write(text)
    return dst


# The timing binary (oracle/_ref/tis_ref_bench): the same patched engine built
# as the CPU baseline is timed, -O3 and with glibc's own rand() (no shim); the
# harness's --rng philox is then ignored.  The parity binary (tis_ref) keeps -O2
# and the shim.
BENCH_FLAGS = ["-O3", "-ffp-contract=off", "-fno-fast-math"]


def _compile_all(jobs, verbose):
    from concurrent.futures import ThreadPoolExecutor

    def run(c):
        if verbose:
            print(" ".join(c))
        subprocess.run(c, check=True)

    with ThreadPoolExecutor(max_workers=len(jobs)) as ex:
        list(ex.map(run, jobs))


def build(verbose=False, bench=False):
    """Returns the path of oracle/_ref/tis_ref (bench=True: oracle/_ref/tis_ref_bench),
    or None when no source is available.  Both binaries are (re)built together."""
    src = reference_source()
    patched = os.path.join(OUT, "engine_patched.cpp")
    if src is not None:
        patched = make_patched_copy(src)
    elif not os.path.isfile(patched):
        return None
    exe = os.path.join(OUT, "tis_ref")
    exe_b = os.path.join(OUT, "tis_ref_bench")
    if os.path.isfile(exe) and os.path.isfile(exe_b) and \
            min(os.path.getmtime(exe), os.path.getmtime(exe_b)) > max(
                os.path.getmtime(patched), os.path.getmtime(os.path.join(HERE, "ref_harness.cpp"))):
        return exe_b if bench else exe
    common = ["g++", "-O2", "-ffp-contract=off", "-fno-fast-math", "-w", "-I", HERE]
    common_b = ["g++", *BENCH_FLAGS, "-w", "-I", HERE]
    mpi = ["-I", os.path.join(HERE, "mpi_stub")]
    eng_o = os.path.join(OUT, "engine.o")
    eng_b = os.path.join(OUT, "engine_bench.o")
    har_o = os.path.join(OUT, "harness.o")
    har_b = os.path.join(OUT, "harness_bench.o")
    _compile_all([
        common + mpi + ["-include", os.path.join(HERE, "ref_rng_shim.h"), "-Dmain=tis_ref_main", "-c", patched,
                        "-o", eng_o],
        common_b + mpi + ["-Dmain=tis_ref_main", "-c", patched, "-o", eng_b],
        common + ["-c", os.path.join(HERE, "ref_harness.cpp"), "-o", har_o],
        common_b + ["-c", os.path.join(HERE, "ref_harness.cpp"), "-o", har_b],
    ], verbose)
    _compile_all([["g++", eng_o, har_o, "-o", exe, "-lm"], ["g++", eng_b, har_b, "-o", exe_b, "-lm"]], verbose)
    return exe_b if bench else exe


EXPORTER_REL = os.path.join("analysis", "make_ninfo", "16SCD_ninfo.cpp")


def build_exporter(verbose=False):
    """The reference's topology exporter (analysis/make_ninfo/16SCD_ninfo.cpp, which
    writes 16SCD_ninfo.ninfo, .psf and .cg.pdb from the four input files in its
    working directory) compiled unmodified from where it lies, with the single-rank
    MPI stub, into oracle/_ref/tis_ref_exporter.  Returns its path, or None when the
    reference is absent (the exporter pins are CPU tests of this container)."""
    roots = [os.environ.get("TIS_REFERENCE_ROOT"), "/root/reference"]
    src = next((os.path.join(r, EXPORTER_REL) for r in roots if r and os.path.isfile(os.path.join(r, EXPORTER_REL))),
               None)
    if src is None:
        return None
    os.makedirs(OUT, exist_ok=True)
    exe = os.path.join(OUT, "tis_ref_exporter")
    if os.path.isfile(exe) and os.path.getmtime(exe) > os.path.getmtime(src):
        return exe
    cmd = ["g++", "-O2", "-ffp-contract=off", "-w", "-include", os.path.join(HERE, "mpi_stub", "mpi.h"), src, "-o",
           exe, "-lm"]
    if verbose:
        print(" ".join(cmd))
    subprocess.run(cmd, check=True)
    return exe


if __name__ == "__main__":
    p = build(verbose="-v" in sys.argv)
    print(p if p else "reference source not available; oracle/_ref not built")
