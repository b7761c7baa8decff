"""Build the CUDA library in-tree: tmc_gb300/libtmc_gb300.so (sm_103a only).

Each translation unit compiles in parallel with `nvcc -c`, then one link step.  The library is
compiled with -fmad=false (device code) and -ffp-contract=off (host code): the kernels restate the
reference's CPU arithmetic operation by operation, and fused multiply-adds would round differently;
hot loops that want FMAs use explicit intrinsics.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
OUT = os.path.join(HERE, "libtmc_gb300.so")
BUILD = os.path.join(HERE, "_build")
SOURCES = ["runtime.cu", "dmc_front.cu", "dmc_mesh.cu", "tmc_cells.cu", "halfedges.cu", "scan.cu", "count_static.cu", "server.cu", "volume_io.cu", "mesh_stats.cu"]
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
FLAGS = ["-std=c++17", "-O3", "-lineinfo", "-fmad=false", "-Xcompiler", "-fPIC", "-Xcompiler", "-ffp-contract=off",
         "--expt-relaxed-constexpr", "-diag-suppress", "177"]


def nvcc():
    p = shutil.which("nvcc")
    if p:
        return p
    cand = "/usr/local/cuda/bin/nvcc"
    if os.path.exists(cand):
        return cand
    raise RuntimeError("nvcc not found")


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    deps.append(os.path.join(os.path.dirname(HERE), "include", "tmc_gb300.h"))
    return any(os.path.getmtime(d) > t for d in deps)


def build(force: bool = False, verbose: bool = False) -> str:
    os.makedirs(BUILD, exist_ok=True)
    cc = nvcc()
    jobs = []
    objs = []
    for src in SOURCES:
        s = os.path.join(CSRC, src)
        if not os.path.exists(s):
            continue
        o = os.path.join(BUILD, src.replace(".cu", ".o"))
        objs.append(o)
        if force or _stale(o, s):
            jobs.append([cc, *ARCH, *FLAGS, "-c", s, "-o", o])
    if jobs:
        with cf.ThreadPoolExecutor(max_workers=min(8, len(jobs))) as ex:
            for cmd, r in zip(jobs, ex.map(lambda c: subprocess.run(c, capture_output=True, text=True), jobs)):
                if r.returncode != 0:
                    raise RuntimeError("nvcc failed: " + " ".join(cmd) + "\n" + r.stdout + r.stderr)
                if verbose and (r.stdout or r.stderr):
                    print(r.stdout + r.stderr, file=sys.stderr)
    if jobs or not os.path.exists(OUT):
        cmd = [cc, *ARCH, "-shared", "-o", OUT, *objs, "-lcudart"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed: " + r.stdout + r.stderr)
    return OUT


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
