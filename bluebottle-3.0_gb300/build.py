"""Build the in-tree CUDA libraries of the package for sm_103a.

    python build.py            # libbbpp.so (+ libbbpp_bluebottle.so)
    python build.py --check    # compile only, report registers / spills

Each translation unit is compiled in parallel with
`nvcc -gencode arch=compute_103a,code=sm_103a -lineinfo -O3`, then linked into
bbpp/_lib/.  Nothing is installed into site-packages.
"""
import argparse
import concurrent.futures as cf
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
LIB = os.path.join(HERE, "bbpp", "_lib")
OBJ = os.path.join(HERE, "_build")
INC = os.path.join(os.path.dirname(HERE), "include")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
NVFLAGS = ["-O3", "-lineinfo", "-std=c++17", "-Xcompiler", "-fPIC", "--expt-relaxed-constexpr",
           "-I", INC, "-I", CSRC]

CORE = ["bbpp_solver.cu", "bbpp_ir.cu", "bbpp_net.cu", "bbpp_noalloc.cu", "bbpp_tma.cu"]
DROPIN = ["bbpp_bluebottle.cu"]


def nvcc():
    p = shutil.which("nvcc") or "/usr/local/cuda/bin/nvcc"
    return p


def compile_one(src, verbose):
    out = os.path.join(OBJ, os.path.splitext(src)[0] + ".o")
    srcp = os.path.join(CSRC, src)
    deps = [srcp] + [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".cuh", ".h"))]
    deps.append(os.path.join(INC, "bbpp.h"))
    if os.path.exists(out) and all(os.path.getmtime(out) >= os.path.getmtime(d) for d in deps if os.path.exists(d)):
        return out, ""
    cmd = [nvcc()] + ARCH + NVFLAGS + ["-c", srcp, "-o", out]
    if verbose:
        cmd += ["-Xptxas", "-v"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("nvcc failed for %s:\n%s\n%s" % (src, r.stdout, r.stderr))
    return out, r.stderr


def link(objs, name, extra=()):
    os.makedirs(LIB, exist_ok=True)
    out = os.path.join(LIB, name)
    cmd = [nvcc()] + ARCH + ["-shared", "-o", out] + list(objs) + list(extra) + ["-lcudart"]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed for %s:\n%s\n%s" % (name, r.stdout, r.stderr))
    return out


def build(verbose=False):
    os.makedirs(OBJ, exist_ok=True)
    srcs = CORE + [s for s in DROPIN if os.path.exists(os.path.join(CSRC, s))]
    with cf.ThreadPoolExecutor(max_workers=max(2, min(8, os.cpu_count() or 2))) as ex:
        res = dict(zip(srcs, ex.map(lambda s: compile_one(s, verbose), srcs)))
    if verbose:
        for s, (_, log) in res.items():
            if log:
                sys.stderr.write("== %s\n%s\n" % (s, log))
    core = link([res[s][0] for s in CORE], "libbbpp.so")
    outs = [core]
    dsrc = [s for s in DROPIN if s in res]
    if dsrc:
        outs.append(link([res[s][0] for s in dsrc], "libbbpp_bluebottle.so",
                         ["-L" + LIB, "-lbbpp", "-Xlinker", "-rpath=$ORIGIN"]))
    return outs


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--check", action="store_true")
    a = ap.parse_args()
    for o in build(verbose=a.check):
        print(o)
