"""Build libnqs_gb300.so (sm_103a) in-tree with nvcc.

Each translation unit is compiled in parallel (one -gencode, no cmake), then
linked into spin_based_neural_network_gb300/libnqs_gb300.so.  Only the CUDA
runtime and the driver library are linked; no torch, no cuBLAS.
"""
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

PKG = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(PKG)
CSRC = os.path.join(PKG, "csrc")
BUILD = os.path.join(PKG, "_build")
LIB = os.path.join(PKG, "libnqs_gb300.so")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
SOURCES = ["nqs_context.cu", "nqs_ansatz.cu", "nqs_local_energy.cu", "nqs_sampler.cu", "nqs_sr.cu",
           "nqs_mixed.cu", "nqs_made.cu", "nqs_batch.cu", "nqs_ed.cu", "nqs_mlp_tc.cu"]


def nvcc():
    cand = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    if not os.path.exists(cand):
        raise RuntimeError("nvcc not found: the CUDA toolkit is required to build libnqs_gb300.so")
    return cand


def flags():
    return ARCH + ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC,-O2",
                   "-I" + os.path.join(ROOT, "include"), "-I" + CSRC]


def _stale(obj, src):
    if not os.path.exists(obj):
        return True
    t = os.path.getmtime(obj)
    deps = [src] + [os.path.join(CSRC, h) for h in os.listdir(CSRC) if h.endswith(".cuh")]
    deps += [os.path.join(ROOT, "include", "nqs", h) for h in os.listdir(os.path.join(ROOT, "include", "nqs"))]
    return any(os.path.getmtime(d) > t for d in deps)


def build(verbose=False, extra=()):
    os.makedirs(BUILD, exist_ok=True)
    nv = nvcc()
    jobs = []
    for s in SOURCES:
        src = os.path.join(CSRC, s)
        obj = os.path.join(BUILD, s.replace(".cu", ".o"))
        if _stale(obj, src):
            jobs.append([nv] + flags() + list(extra) + ["-c", src, "-o", obj])
    def run(cmd):
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("nvcc failed:\n" + " ".join(cmd) + "\n" + r.stdout + r.stderr)
        if verbose and (r.stdout or r.stderr):
            sys.stderr.write(r.stdout + r.stderr)
    with cf.ThreadPoolExecutor(max_workers=min(8, os.cpu_count() or 4)) as ex:
        list(ex.map(run, jobs))
    objs = [os.path.join(BUILD, s.replace(".cu", ".o")) for s in SOURCES]
    if jobs or not os.path.exists(LIB) or any(os.path.getmtime(o) > os.path.getmtime(LIB) for o in objs):
        cmd = [nv] + ARCH + ["-shared", "-o", LIB] + objs + ["-lcuda"]
        r = subprocess.run(cmd, capture_output=True, text=True)
        if r.returncode != 0:
            raise RuntimeError("link failed:\n" + r.stdout + r.stderr)
    return LIB


if __name__ == "__main__":
    print(build(verbose=True))
