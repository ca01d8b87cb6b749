"""Build recipe of the native library and the drop-in executable (sm_103a only).

Outputs, in-tree under pandemicthrust_gb300/_build/ (git-ignored):
  libpandemic_gb300.so   the C-ABI library declared in include/pandemic_gb300.h
  pt_sim                 drop-in executable: constants.csv + seed.txt in the working
                         directory -> output_infected_stats.csv, output_rn.csv,
                         infected_max.txt, profile_log.csv (the reference's file contract)
  pt_batch               batch driver: every experiment of a PythonBatcher
                         experiment_files.txt (x seeds) as one batch
Translation units compile in parallel; the whole build takes well under a minute.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(HERE)
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "_build")
INCLUDE = os.path.join(ROOT, "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
LIB = os.path.join(OUT, "libpandemic_gb300.so")
CLI = os.path.join(OUT, "pt_sim")
BATCH_CLI = os.path.join(OUT, "pt_batch")

CUDA_SOURCES = ["pt_kernels.cu", "pt_static_table.cu", "pt_mlp.cu"]
HOST_SOURCES = ["pt_sim.cpp", "pt_host.cpp"]


def _nvcc():
    for cand in (os.environ.get("NVCC"), "/usr/local/cuda/bin/nvcc", "nvcc"):
        if cand and (os.path.sep not in cand or os.path.exists(cand)):
            return cand
    return "nvcc"


def _sources_mtime():
    files = [os.path.join(CSRC, f) for f in os.listdir(CSRC)] + [os.path.join(INCLUDE, f) for f in os.listdir(INCLUDE)]
    return max(os.path.getmtime(f) for f in files)


def build(verbose=False, force=False):
    os.makedirs(OUT, exist_ok=True)
    outputs = (LIB, CLI, BATCH_CLI)
    if not force and all(os.path.exists(f) for f in outputs) and \
            min(os.path.getmtime(f) for f in outputs) >= _sources_mtime():
        return LIB
    nvcc = _nvcc()
    common = ["-std=c++17", "-O3", "-I", INCLUDE, "-I", CSRC, "-Xcompiler", "-fPIC"]
    jobs = []
    objs = []
    for src in CUDA_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        cmd = [nvcc] + ARCH + common + ["-lineinfo", "-Xptxas", "-v" if verbose else "-O3",
                                        "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append(cmd)
    for src in HOST_SOURCES:
        obj = os.path.join(OUT, src + ".o")
        objs.append(obj)
        cmd = [nvcc] + common + ["-Xcompiler", "-ffp-contract=off", "-c", os.path.join(CSRC, src), "-o", obj]
        jobs.append(cmd)
    procs = []
    for cmd in jobs:
        if verbose:
            print(" ".join(cmd))
        procs.append(subprocess.Popen(cmd))
    bad = [p.args for p in procs if p.wait() != 0]
    if bad:
        raise RuntimeError("compile failed: %s" % bad[0])
    link = [nvcc] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
    if verbose:
        print(" ".join(link))
    subprocess.check_call(link)
    # the executables: the drop-in pt_sim and the batch driver, both over the library
    cli_objs = {}
    procs = []
    for src in ("pt_cli.cpp", "pt_batch_cli.cpp", "pt_output.cpp"):
        obj = os.path.join(OUT, src + ".o")
        cli_objs[src] = obj
        procs.append(subprocess.Popen([nvcc] + common + ["-Xcompiler", "-ffp-contract=off", "-c",
                                                         os.path.join(CSRC, src), "-o", obj]))
    bad = [p.args for p in procs if p.wait() != 0]
    if bad:
        raise RuntimeError("compile failed: %s" % bad[0])
    for exe, main_src in ((CLI, "pt_cli.cpp"), (BATCH_CLI, "pt_batch_cli.cpp")):
        subprocess.check_call([nvcc] + ARCH + ["-o", exe, cli_objs[main_src], cli_objs["pt_output.cpp"], "-L", OUT,
                                               "-lpandemic_gb300", "-Xlinker", "-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(verbose="-v" in sys.argv, force=True))
