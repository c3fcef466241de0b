"""Build oracle/_ref/ref_solver.cubin: the reference's unmodified
src/solver_kernel.cu (from the reference tree) plus ref_kernels.cu, for
sm_103a, and oracle/_ref/ref_cages.cubin: its src/particle_kernel.cu (the
cage builder's kernels) plus ref_cages_kernels.cu, so that the reference's
own CUDA kernels can run on the GPU machine, where the reference tree is absent.  Test and measurement infrastructure;
nothing of the reference is written into the repository (the cubin goes to
the git-ignored oracle/_ref).
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
OUT = os.path.join(os.path.dirname(HERE), "_ref")
sys.path.insert(0, os.path.dirname(HERE))
import refpath  # noqa: E402

REF = refpath.tree()
SRC = refpath.src()
SHIM = os.path.join(HERE, "shim")


def build(quiet=False):
    if not os.path.isfile(os.path.join(SRC, "solver_kernel.cu")):
        if not quiet:
            print("reference tree not found at", REF)
        return None
    os.makedirs(OUT, exist_ok=True)
    out = os.path.join(OUT, "ref_solver.cubin")
    nvcc = os.environ.get("NVCC", "nvcc")
    # the shim directory supplies a one-rank mpi.h for the reference headers
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-DDOUBLE", "-DJACOBI",
           "-w", "-I", SHIM, "-I", SRC, "-o", out, os.path.join(HERE, "ref_kernels.cu")]
    subprocess.run(cmd, check=True)
    # the reference's cage kernels (src/particle_kernel.cu), without FMA
    # contraction: the arithmetic of the host pin the cage fixtures come from
    cages = os.path.join(OUT, "ref_cages.cubin")
    cmd = [nvcc, "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-fmad=false", "-DDOUBLE",
           "-DJACOBI", "-w", "-I", SHIM, "-I", SRC, "-I", HERE, "-o", cages, os.path.join(HERE, "ref_cages_kernels.cu")]
    subprocess.run(cmd, check=True)
    return out


if __name__ == "__main__":
    p = build()
    sys.exit(0 if p else 1)
