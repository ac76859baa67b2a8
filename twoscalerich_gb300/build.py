"""Build step of the GB300 library: compiles the CUDA kernels and the host
C++ of ``twoscalerich_gb300/csrc`` into ``twoscalerich_gb300/libtsr_gb300.so``
(in tree, for sm_103a only) with nvcc.

Translation units compile in parallel; the whole build takes well under a
minute.  Device code is compiled with ``-fmad=false`` and host code with
``-ffp-contract=off``: the library's floating-point results are defined
operation by operation, and no multiply-add may be fused that the source
does not fuse explicitly.
"""
import concurrent.futures as cf
import os
import platform
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libtsr_gb300.so")

CUDA_HOME = os.environ.get("CUDA_HOME", "/usr/local/cuda")
NVCC = os.path.join(CUDA_HOME, "bin", "nvcc")
ARCH = ["-gencode", "arch=compute_103a,code=sm_103a"]
CU_SOURCES = ["tsr_kernels.cu", "tsr_ctx.cu", "tsr_noalloc.cu", "tsr_mlp.cu", "tsr_homog.cu", "tsr_meshdev.cu"]
CPP_SOURCES = ["tsr_host.cpp", "tsr_dropin.cpp"]


def _nvcc():
    if os.path.exists(NVCC):
        return NVCC
    found = shutil.which("nvcc")
    if not found:
        raise RuntimeError("nvcc not found: the GB300 library cannot be built")
    return found


def _run(cmd):
    r = subprocess.run(cmd, stdout=subprocess.PIPE, stderr=subprocess.STDOUT, text=True)
    if r.returncode != 0:
        raise RuntimeError("build command failed:\n%s\n%s" % (" ".join(cmd), r.stdout))
    return r.stdout


def _sources_newer(target, sources):
    if not os.path.exists(target):
        return True
    t = os.path.getmtime(target)
    return any(os.path.getmtime(s) > t for s in sources)


def build(verbose=False, force=False):
    os.makedirs(BUILD, exist_ok=True)
    nvcc = _nvcc()
    headers = [os.path.join(CSRC, f) for f in os.listdir(CSRC) if f.endswith((".h", ".cuh"))]
    headers += [os.path.join(HERE, "..", "include", f)
                for f in os.listdir(os.path.join(HERE, "..", "include"))]
    # OpenMP: the host evaluates independent phi_1 Pade approximants of an
    # Arnoldi batch side by side
    host_flags = ["-fPIC", "-O2", "-ffp-contract=off", "-fopenmp"]
    if platform.machine() == "x86_64":
        # fma() as the hardware instruction (a library call otherwise); the
        # results are the same either way, fma rounds once
        host_flags.append("-mfma")
    jobs = []
    objs = []
    for src in CU_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _sources_newer(o, [s] + headers):
            cmd = [nvcc, "-c", s, "-o", o, "-O3", "-std=c++17", "-lineinfo", "-fmad=false",
                   "-Xptxas", "-v" if verbose else "-O3"] + ARCH
            for f in host_flags:
                cmd += ["-Xcompiler", f]
            jobs.append(cmd)
    for src in CPP_SOURCES:
        s = os.path.join(CSRC, src)
        o = os.path.join(BUILD, src + ".o")
        objs.append(o)
        if force or _sources_newer(o, [s] + headers):
            cmd = [nvcc, "-c", s, "-o", o, "-O2", "-std=c++17"]
            for f in host_flags:
                cmd += ["-Xcompiler", f]
            jobs.append(cmd)
    with cf.ThreadPoolExecutor(max_workers=max(1, min(len(jobs), os.cpu_count() or 1))) as ex:
        outs = list(ex.map(_run, jobs))
    if verbose:
        for o in outs:
            sys.stdout.write(o)
    if force or jobs or not os.path.exists(LIB):
        _run([nvcc, "-shared", "-o", LIB] + objs + ["-cudart", "static", "-lgomp"] + ARCH)
    return LIB


def build_oracle(reference_root=None):
    """Build the CPU oracle (always) and, when the reference tree is
    present, the library compiled from the reference's own sources (the
    tree is reference_root, else TSR_REFERENCE_ROOT, else the oracle
    recipe's default)."""
    oracle_dir = os.path.join(HERE, "..", "oracle")
    _run(["make", "-s", "-C", oracle_dir, "oracle"])
    cmd = ["make", "-s", "-C", oracle_dir, "ref-if-present"]
    if reference_root:
        cmd.append("REF=%s" % reference_root)
    _run(cmd)


if __name__ == "__main__":
    build(verbose="-v" in sys.argv, force="-f" in sys.argv)
    build_oracle()
    print(LIB)
