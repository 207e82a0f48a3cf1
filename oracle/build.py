"""Build recipe for the test oracle -- TEST INFRASTRUCTURE ONLY.

* ``oracle/_build/liboracle.so``: the C++ restatement (prbf_oracle.cpp), built on every
  machine (plain g++, OpenMP, -ffp-contract=off so expressions round as written).
* ``oracle/_ref/libref2d.so`` / ``libref3d.so``: the reference's own 2d/ and 3d/ sources
  (get_cluster.h, get_trunc.h, get_buffer.h, get_vorticity.h, matmult.cxx,
  mpi_range.cxx) compiled unmodified where they lie, against the sequential PETSc/MPI
  stand-in in ``oracle/ref_stub``. Only built where the reference tree is present; it
  generates the golden fixtures under tests/golden and is never shipped or linked by
  the product.
* ``oracle/_ref/gpumatmult_2d.cubin`` / ``_3d.cubin``: the reference's own FP32 GPU kernel
  (2d/gpumatmult.cu, 3d/gpumatmult.cu), device code compiled unmodified for sm_103a where
  the reference tree is present; ``oracle/refgpu.py`` loads it through the CUDA driver API
  for the seam's parity test.
"""
import os
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
# Where the reference's sources are read from: $PETRBF_REFERENCE_TREE, else the read-only
# checkout this recipe was written against. Absent on machines that only run the tests.
REFERENCE_TREE_DEFAULT = "/root/reference"


def reference_tree():
    """The reference checkout to compile from, or None where there is none."""
    root = os.environ.get("PETRBF_REFERENCE_TREE", REFERENCE_TREE_DEFAULT)
    return root if os.path.isdir(root) else None
CXXFLAGS = ["-O3", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-fopenmp"]


def _run(cmd):
    r = subprocess.run(cmd, capture_output=True, text=True)
    if r.returncode != 0:
        raise RuntimeError("build failed: %s\n%s%s" % (" ".join(cmd), r.stdout, r.stderr))


def _stale(out, srcs):
    if not os.path.exists(out):
        return True
    t = os.path.getmtime(out)
    return any(os.path.getmtime(s) > t for s in srcs)


def _host_flags():
    """x86-64 builds call std::fma through libm unless FMA instructions are enabled; the
    Arm target has them in its base ISA. fma rounds once on both, so results are equal."""
    import platform
    if platform.machine() in ("x86_64", "AMD64"):
        try:
            with open("/proc/cpuinfo") as fh:
                if " fma " in fh.read():
                    return ["-mfma"]
        except OSError:
            pass
    return []


def build_oracle(force=False):
    out = os.path.join(HERE, "_build", "liboracle.so")
    srcs = [os.path.join(HERE, "prbf_oracle.cpp"), os.path.join(HERE, "prbf_oracle.h")]
    if force or _stale(out, srcs):
        os.makedirs(os.path.dirname(out), exist_ok=True)
        _run(["g++"] + CXXFLAGS + _host_flags() + ["-o", out, srcs[0]])
    return out


def build_ref(ref_root, force=False):
    """Compile the reference's own sources (read in place) into oracle/_ref."""
    outs = []
    stub = os.path.join(HERE, "ref_stub")
    for dim in (2, 3):
        tree = os.path.join(ref_root, "%dd" % dim)
        if not os.path.isdir(tree):
            continue
        out = os.path.join(HERE, "_ref", "libref%dd.so" % dim)
        srcs = [os.path.join(HERE, "ref_driver.cpp"), os.path.join(tree, "matmult.cxx"),
                os.path.join(tree, "mpi_range.cxx")]
        deps = srcs + [os.path.join(stub, "petscksp.h"), os.path.join(stub, "mpi.h")]
        if force or _stale(out, deps):
            os.makedirs(os.path.dirname(out), exist_ok=True)
            _run(["g++", "-O2", "-std=c++17", "-fPIC", "-shared", "-ffp-contract=off", "-w",
                  "-DREF_DIM=%d" % dim, "-I", stub, "-I", tree, "-o", out] + srcs)
        outs.append(out)
        # the reference's own FP32 GPU kernel (gpumatmult.cu), device code only, unmodified
        cu = os.path.join(tree, "gpumatmult.cu")
        cub = os.path.join(HERE, "_ref", "gpumatmult_%dd.cubin" % dim)
        if os.path.exists(cu) and (force or _stale(cub, [cu])):
            _run(["nvcc", "-cubin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3", "-w", "-o", cub, cu])
        if os.path.exists(cub):
            outs.append(cub)
    return outs


if __name__ == "__main__":
    print(build_oracle(force="-f" in sys.argv))
    if len(sys.argv) > 1 and os.path.isdir(sys.argv[-1]):
        print(build_ref(sys.argv[-1], force="-f" in sys.argv))
