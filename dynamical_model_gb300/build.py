"""Build libmoloch_gb300.so in-tree for sm_103a.

Translation units compiled in parallel:
  csrc/moloch_kernels_exact.cu  nvcc, FP64, --fmad=false (reference evaluation order)
  csrc/moloch_kernels_fast.cu   nvcc, FP64 + FP32, multiply-add contraction allowed
  csrc/moloch_persist.cu        nvcc, the persistent ensemble kernel (contraction allowed)
  csrc/moloch_noalloc.cu        nvcc, FP64, --fmad=false (allocation-free WAF entry point)
  csrc/moloch_mlp.cu            nvcc, tcgen05 GEMM and the surrogate MLP kernels
  csrc/moloch_api.cpp           host C ABI, -ffp-contract=off
  csrc/moloch_ideal.cpp         host idealized-state generator, -ffp-contract=off
"""
import os
import shutil
import subprocess
import sys

HERE = os.path.dirname(os.path.abspath(__file__))
CSRC = os.path.join(HERE, "csrc")
BUILD = os.path.join(HERE, "_build")
LIB = os.path.join(HERE, "libmoloch_gb300.so")
ARCH = "-gencode=arch=compute_103a,code=sm_103a"


def _cuda_home():
    for cand in (os.environ.get("CUDA_HOME"), "/usr/local/cuda"):
        if cand and os.path.exists(os.path.join(cand, "bin", "nvcc")):
            return cand
    nvcc = shutil.which("nvcc")
    if nvcc:
        return os.path.dirname(os.path.dirname(nvcc))
    raise RuntimeError("nvcc not found")


def _sources():
    return [os.path.join(CSRC, f) for f in sorted(os.listdir(CSRC))
            if f.endswith((".cu", ".cuh", ".cpp", ".h"))] + [
        os.path.join(os.path.dirname(HERE), "include", "moloch_gb300.h")]


def _stale():
    if not os.path.exists(LIB):
        return True
    t = os.path.getmtime(LIB)
    return any(os.path.getmtime(s) > t for s in _sources())


def build(force=False, verbose=False):
    """Compile and link; returns the path of the shared library."""
    if not force and not _stale():
        return LIB
    cuda = _cuda_home()
    nvcc = os.path.join(cuda, "bin", "nvcc")
    os.makedirs(BUILD, exist_ok=True)
    inc = ["-I" + os.path.join(cuda, "include"), "-I" + CSRC]
    nv_common = [nvcc, "-std=c++17", ARCH, "-O3", "-lineinfo", "-Xcompiler", "-fPIC",
                 "-Xcompiler", "-ffp-contract=off", "-Xptxas", "-warn-spills"] + inc
    jobs = [
        nv_common + ["--fmad=false", "-c", os.path.join(CSRC, "moloch_kernels_exact.cu"),
                     "-o", os.path.join(BUILD, "kexact.o")],
        nv_common + ["-c", os.path.join(CSRC, "moloch_kernels_fast.cu"),
                     "-o", os.path.join(BUILD, "kfast.o")],
        nv_common + ["-c", os.path.join(CSRC, "moloch_persist.cu"), "-o", os.path.join(BUILD, "persist.o")],
        nv_common + ["--fmad=false", "-c", os.path.join(CSRC, "moloch_noalloc.cu"),
                     "-o", os.path.join(BUILD, "noalloc.o")],
        nv_common + ["-c", os.path.join(CSRC, "moloch_mlp.cu"), "-o", os.path.join(BUILD, "mlp.o")],
        nv_common + ["--fmad=false", "-c", os.path.join(CSRC, "moloch_init.cu"), "-o", os.path.join(BUILD, "init.o")],
        ["g++", "-std=c++17", "-O2", "-fPIC", "-pthread", "-ffp-contract=off", "-fno-fast-math"] + inc +
        ["-c", os.path.join(CSRC, "moloch_api.cpp"), "-o", os.path.join(BUILD, "api.o")],
        ["g++", "-std=c++17", "-O2", "-fPIC", "-ffp-contract=off", "-fno-fast-math"] + inc +
        ["-c", os.path.join(CSRC, "moloch_ideal.cpp"), "-o", os.path.join(BUILD, "ideal.o")],
    ]
    procs = [(j, subprocess.Popen(j, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)) for j in jobs]
    failed = []
    for j, p in procs:
        out = p.communicate()[0].decode(errors="replace")
        if p.returncode != 0:
            failed.append((j, out))
        elif verbose and out.strip():
            print(out)
    if failed:
        msg = "\n".join(" ".join(j) + "\n" + out for j, out in failed)
        raise RuntimeError("build failed:\n" + msg)
    tmp = LIB + ".tmp"
    link = [nvcc, ARCH, "-shared", "-o", tmp] + [os.path.join(BUILD, o) for o in
                                                 ("kexact.o", "kfast.o", "persist.o", "noalloc.o", "mlp.o", "init.o", "api.o", "ideal.o")] + ["-lcudart", "-Xcompiler", "-pthread"]
    r = subprocess.run(link, stdout=subprocess.PIPE, stderr=subprocess.STDOUT)
    if r.returncode != 0:
        raise RuntimeError("link failed:\n" + r.stdout.decode(errors="replace"))
    os.replace(tmp, LIB)
    return LIB


if __name__ == "__main__":
    print(build(force="--force" in sys.argv, verbose=True))
