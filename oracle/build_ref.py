"""Build the reference-derived checker ``oracle/_ref/libptref.so`` (test infrastructure).

The reference's simulation kernels are plain C++ inside ``__global__``/``__device__``
functions, so the hot-path slices of PandemicThrust/PandemicThrust/PandemicSim.cu
compile for the host once the CUDA qualifiers are defined away.  This script copies
the cited line ranges, verbatim and in order, into a temporary include file (deleted
after the build: reference source never enters the repository) and compiles them
with ``oracle/ref_harness.cpp``, which restates the host flow of ``class
PandemicSim`` around them, plus the reference's own ``host_functions.cpp``.  Only
the shared library ``oracle/_ref/libptref.so`` is kept.

Run here, where the reference tree exists:  python oracle/build_ref.py
The GPU test box has no reference tree; the tests that need this library skip there.
"""
import os
import shutil
import subprocess
import sys
import tempfile

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(HERE, "_ref")
# The reference checkout: PT_REFERENCE_ROOT, else a directory named "reference" beside
# this repository's root.
REF_ROOT = os.environ.get("PT_REFERENCE_ROOT") or os.path.join(os.path.dirname(os.path.dirname(HERE)), "reference")
SRC_DIR = os.path.join(REF_ROOT, "PandemicThrust", "PandemicThrust")
R123_DIR = os.path.join(REF_ROOT, "PandemicThrust", "Random123")

# (file, first line, last line, what it holds); inclusive, 1-based.
SLICES = [
    ("PandemicSim.h", 283, 302, "day-of-week and status macros"),
    ("PandemicSim.h", 304, 437, "device/kernel prototypes"),
    ("PandemicSim.cu", 26, 96, "constant tables and pointer structs"),
    ("PandemicSim.cu", 268, 566, "PandemicSim::setup_loadParameters"),
    ("PandemicSim.cu", 569, 701, "PandemicSim::setup_pushDeviceData"),
    ("PandemicSim.cu", 971, 1044, "weekend errand generation and fishing"),
    ("PandemicSim.cu", 1127, 1162, "PandemicSim::setup_scaleSimulation"),
    ("PandemicSim.cu", 1642, 1665, "n_unique_numbers, roundHalfUp_toInt"),
    ("PandemicSim.cu", 1669, 2094, "contacts, location lookups, weekend schedule kernel"),
    ("PandemicSim.cu", 2097, 2192, "kernel_countInfectedStatusAndRecover"),
    ("PandemicSim.cu", 2307, 2531, "infection probability, household/workplace setup kernels"),
    ("PandemicSim.cu", 2534, 2549, "household count functors"),
    ("PandemicSim.cu", 2828, 2862, "setup_calculateInfectionData, setup_loadSeed"),
    ("PandemicSim.cu", 2909, 3022, "weekday schedule kernel"),
    ("PandemicSim.cu", 3048, 3379, "infection: claim, process contacts, day kernels"),
    ("PandemicSim.cu", 3492, 3511, "device_getWorkplaceMaxContacts"),
    ("PandemicSim.cu", 3579, 3605, "hh_peopleCount_functor"),
    ("PandemicSim.cu", 3667, 3705, "weekday errand regeneration"),
    ("PandemicSim.cu", 3742, 3778, "weekend errand regeneration, assignWorkplaceFunctor"),
    ("PandemicSim.cu", 3872, 3890, "device_recalcWorkplace"),
    ("PandemicSim.cu", 3974, 3988, "device_getInfectionProfile"),
]


def write_slices(path):
    parts = ["/* generated by oracle/build_ref.py from the reference tree; do not commit */\n"]
    for fname, a, b, what in SLICES:
        full = os.path.join(SRC_DIR, fname)
        with open(full, encoding="latin-1") as fh:
            lines = fh.read().split("\n")
        if b > len(lines):
            raise SystemExit(f"{fname} has {len(lines)} lines, slice ends at {b}")
        parts.append(f"/* {fname}:{a}-{b} {what} */\n")
        parts.append(f'#line {a} "{full}"\n')
        parts.append("\n".join(lines[a - 1:b]) + "\n")
    with open(path, "w") as fh:
        fh.write("".join(parts))


def build(verbose=False):
    if not os.path.isdir(SRC_DIR):
        if verbose:
            print("reference tree not present; oracle/_ref not built")
        return None
    os.makedirs(OUT, exist_ok=True)
    stale = os.path.join(OUT, "ref_slices.inc")
    if os.path.exists(stale):
        os.remove(stale)
    tmp = tempfile.mkdtemp(prefix="ptref_")
    try:
        inc = os.path.join(tmp, "ref_slices.inc")
        write_slices(inc)
        so = os.path.join(OUT, "libptref.so")
        cmd = [
            "g++", "-std=c++20", "-O2", "-ffp-contract=off", "-fPIC", "-shared", "-pthread",
            "-w", "-Wno-narrowing",
            "-I", tmp, "-I", R123_DIR, "-I", SRC_DIR, "-I", HERE,
            os.path.join(HERE, "ref_harness.cpp"),
            os.path.join(SRC_DIR, "host_functions.cpp"),
            "-o", so,
        ]
        if verbose:
            print(" ".join(cmd))
        subprocess.check_call(cmd)
    finally:
        shutil.rmtree(tmp, ignore_errors=True)
    return so


if __name__ == "__main__":
    path = build(verbose=True)
    print(path or "skipped")
    sys.exit(0)
