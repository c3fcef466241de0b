"""Host build of the reference pressure solver, used to pin the oracle.

Compiles the unmodified src/cuda_solver.cu, src/solver_kernel.cu,
src/bluebottle_kernel.cu (the post-solve epilogue's kernels) and
src/particle_kernel.cu (the cage builder's kernels) from the reference tree for the CPU, with the shims in oracle/ref/shim (CUDA execution
model as fibers, one-rank MPI, thrust::inner_product) and the harness in
oracle/ref/harness.cpp, into oracle/_ref/libref.so.  Kernel launches
`k<<<grid, block>>>(args);` are rewritten on the fly, while the source streams
into the compiler, to `emu::launch(grid, block, [&]{ k(args); });` -- no
reference source is written to disk.  cuda_solver.cu is compiled with PP_rhs
renamed to the harness's PP_rhs_inject so a given right-hand side can be
injected.

Test infrastructure only; needs the reference tree (oracle/refpath.py says where).
"""
import os
import re
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
sys.path.insert(0, os.path.dirname(HERE))
import refpath  # noqa: E402

REF = refpath.tree()
SRC = refpath.src()
CXX = os.environ.get("CXX", "g++")
FLAGS = ["-O2", "-fPIC", "-std=c++17", "-ffp-contract=off", "-w", "-DDOUBLE", "-DJACOBI",
         "-I", os.path.join(HERE, "shim"), "-I", SRC, "-include", os.path.join(HERE, "shim", "emu_cuda.h")]


def rewrite_launches(text):
    out = []
    i = 0
    pat = re.compile(r"(\w+)\s*<<<")
    while True:
        m = pat.search(text, i)
        if not m:
            out.append(text[i:])
            break
        out.append(text[i:m.start()])
        name = m.group(1)
        j = text.index(">>>", m.end())
        cfg = text[m.end():j]
        k = j + 3
        while text[k].isspace():
            k += 1
        assert text[k] == "(", "launch without arguments near %r" % text[m.start():k + 20]
        depth, p = 0, k
        while True:
            ch = text[p]
            if ch == "(":
                depth += 1
            elif ch == ")":
                depth -= 1
                if depth == 0:
                    break
            p += 1
        args = text[k + 1:p]
        g, b = [s.strip() for s in cfg.split(",")[:2]]
        out.append("emu::launch(%s, %s, [&]{ %s(%s); })" % (g, b, name, args))
        i = p + 1
    return "".join(out)


def shared_arrays(text):
    """`extern __shared__ T name[];` (dynamic shared memory) becomes a static
    array of 65536 elements: the emulation has no launch-sized shared memory."""
    return re.sub(r"extern\s+__shared__\s+(\w+)\s+(\w+)\s*\[\s*\]", r"static \1 \2[1 << 16]", text)


def compile_ref(src, obj, extra=()):
    text = open(os.path.join(SRC, src)).read()
    text = rewrite_launches(shared_arrays(text))
    cmd = [CXX] + FLAGS + list(extra) + ["-x", "c++", "-c", "-", "-o", obj]
    r = subprocess.run(cmd, input=text, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile of %s failed:\n%s" % (src, r.stderr[-6000:]))


def compile_own(src, obj, extra=()):
    cmd = [CXX] + FLAGS + list(extra) + ["-c", os.path.join(HERE, src), "-o", obj]
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("compile of %s failed:\n%s" % (src, r.stderr[-6000:]))


def build():
    if not os.path.isdir(SRC):
        print("reference tree not found (%s); oracle/_ref not built" % SRC)
        return None
    os.makedirs(OUT, exist_ok=True)
    objs = [os.path.join(OUT, n) for n in ("cuda_solver.o", "solver_kernel.o", "harness.o", "emu_runtime.o",
                                           "bluebottle_kernel.o", "particle_kernel.o", "cages_harness.o")]
    compile_ref("cuda_solver.cu", objs[0], ["-DPP_rhs=PP_rhs_inject"])
    compile_ref("solver_kernel.cu", objs[1])
    compile_ref("bluebottle_kernel.cu", objs[4])
    compile_ref("particle_kernel.cu", objs[5])  # the cage kernels of cuda_build_cages
    compile_own("harness.cpp", objs[2])
    compile_own("emu_runtime.cpp", objs[3])
    compile_own("cages_harness.cpp", objs[6])
    lib = os.path.join(OUT, "libref.so")
    r = subprocess.run([CXX, "-shared", "-o", lib] + objs + ["-Wl,--no-undefined", "-lm"], capture_output=True,
                       text=True)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n%s" % r.stderr[-6000:])
    return lib


if __name__ == "__main__":
    print(build())
