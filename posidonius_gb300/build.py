"""Build recipe of the CUDA library (sm_103a, in-tree).

Produces ``posidonius_gb300/_lib/libposidonius_gb300.so`` from the sources in
``posidonius_gb300/csrc`` and the ``posidonius`` command beside it.  The two kernel translation units are compiled
with different contraction settings: ``kernels_exact.cu`` with
``-fmad=false`` (the reference's operation order, no FMA) and
``kernels_fast.cu`` with ``-fmad=true``.
"""
import os
import shutil
import subprocess
import sys
from concurrent.futures import ThreadPoolExecutor

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT_DIR = os.path.join(HERE, "_lib")
LIB = os.path.join(OUT_DIR, "libposidonius_gb300.so")
CLI = os.path.join(OUT_DIR, "posidonius")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
COMMON = ["-O3", "-std=c++17", "-lineinfo", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off"]

UNITS = [
    ("kernels_exact.cu", ["-fmad=false"]),
    ("kernels_fast.cu", ["-fmad=true"]),
    ("ias15_exact.cu", ["-fmad=false"]),
    ("ias15_fast.cu", ["-fmad=true"]),
    ("posi_host.cu", ["-fmad=false"]),
    ("case_reader.cpp", ["-x", "cu", "-fmad=false"]),
    ("diagnostics.cu", ["-fmad=true"]),
    ("snapshot.cpp", ["-x", "cu", "-fmad=false"]),
    ("bincode.cpp", ["-x", "cu", "-fmad=false"]),
    ("adjoint.cu", ["-fmad=true"]),
    ("large.cu", ["-fmad=true"]),
]


def nvcc():
    exe = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(exe):
        raise RuntimeError("nvcc not found")
    return exe


def _sources_newer(target, deps):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(d) > t for d in deps)


def build(force=False, verbose=False, extra_flags=()):
    os.makedirs(OUT_DIR, exist_ok=True)
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".hpp", ".cuh"))]
    headers.append(os.path.join(os.path.dirname(HERE), "include", "posidonius_gb300.h"))
    objs = []
    jobs = []
    for src, flags in UNITS:
        s = os.path.join(CSRC, src)
        o = os.path.join(OUT_DIR, os.path.splitext(src)[0] + ".o")
        objs.append(o)
        if force or _sources_newer(o, [s] + headers):
            cmd = [nvcc()] + ARCH + COMMON + list(flags) + list(extra_flags) + ["-c", s, "-o", o]
            jobs.append(cmd)

    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("compile failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose:
            sys.stdout.write(r.stdout + r.stderr)
        return r

    with ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 2))) as ex:
        list(ex.map(run, jobs))
    if jobs or not os.path.exists(LIB):
        cmd = [nvcc()] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcudart"]
        run(cmd)
    # the `posidonius` command, linked against the library beside it
    cli_src = os.path.join(CSRC, "posi_cli.cpp")
    if force or _sources_newer(CLI, [cli_src, LIB] + headers):
        run([nvcc()] + ARCH + ["-O2", "-std=c++17", "-x", "cu", cli_src, "-o", CLI, "-L" + OUT_DIR,
                               "-lposidonius_gb300", "-lcudart", "-Xlinker", "-rpath,$ORIGIN"])
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose="-v" in sys.argv))
