"""Recipe that builds the reference's own FDK kernels for the GB300.

TEST INFRASTRUCTURE ONLY (golden-fixture generation).

* fatbin: Lukas-kV/TomoKvas FBPG/kernel.cu, compiled where it lies under the
  reference checkout, device code only, sm_103a, with the shim headers of
  oracle/refshim (a stub <windows.h>/<tiffio.h> and a no-op for the removed
  cufftSetCompatibilityMode).  Output: oracle/_ref/tk_ref_kernels.fatbin.
  Needs the reference checkout, so it is built where that exists; the fatbin
  then travels with the repository copy.
* loader: oracle/tk_refrun.cpp -> oracle/_ref/libtk_ref.so (g++, CUDA runtime,
  driver API, cuFFT), built on the machine that runs it.
* rsq reader: FBPG/rsq_load.cpp + oracle/tk_rsqrun.cpp -> oracle/_ref/libtk_rsqref.so
  (g++, CPU only), where the reference checkout exists.
The reference checkout is TK_REFERENCE_DIR (default /root/reference), the CUDA
toolkit CUDA_HOME (default /usr/local/cuda).
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
FATBIN = os.path.join(REF_DIR, "tk_ref_kernels.fatbin")
LOADER = os.path.join(REF_DIR, "libtk_ref.so")
# The reference checkout and the CUDA toolkit: overridable for other machines.
REFERENCE_DIR = os.environ.get("TK_REFERENCE_DIR", "/root/reference")
REFERENCE_KERNEL = os.path.join(REFERENCE_DIR, "FBPG", "kernel.cu")
REFERENCE_RSQ = os.path.join(REFERENCE_DIR, "FBPG", "rsq_load.cpp")
CUDA = os.environ.get("CUDA_HOME", "/usr/local/cuda")
RSQ_LIB = os.path.join(REF_DIR, "libtk_rsqref.so")


def build_fatbin(force: bool = False):
    """Build the fatbin if the reference checkout is present; returns its path or None."""
    if not os.path.exists(REFERENCE_KERNEL):
        return FATBIN if os.path.exists(FATBIN) else None
    os.makedirs(REF_DIR, exist_ok=True)
    if not force and os.path.exists(FATBIN) and os.path.getmtime(FATBIN) >= os.path.getmtime(REFERENCE_KERNEL):
        return FATBIN
    shim = os.path.join(HERE, "refshim")
    cmd = [os.path.join(CUDA, "bin", "nvcc"), "-fatbin", "-gencode", "arch=compute_103a,code=sm_103a", "-O3",
           "-I", shim, "-include", os.path.join(shim, "tk_ref_compat.h"), REFERENCE_KERNEL, "-o", FATBIN,
           "-w"]
    subprocess.run(cmd, check=True)
    return FATBIN


def build_loader(force: bool = False) -> str:
    os.makedirs(REF_DIR, exist_ok=True)
    src = os.path.join(HERE, "tk_refrun.cpp")
    if not force and os.path.exists(LOADER) and os.path.getmtime(LOADER) >= os.path.getmtime(src):
        return LOADER
    tmp = LOADER + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", src, "-I", os.path.join(CUDA, "include"),
           "-L", os.path.join(CUDA, "lib64"), "-L", os.path.join(CUDA, "lib64", "stubs"),
           "-lcudart", "-lcufft", "-lcuda", "-Wl,-rpath," + os.path.join(CUDA, "lib64"), "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, LOADER)
    return LOADER


def build_rsq(force: bool = False):
    """The reference's rsq reader (FBPG/rsq_load.cpp, compiled where it lies, with the Linux stand-ins of
    refshim/tk_rsq_compat.h) and oracle/tk_rsqrun.cpp -> oracle/_ref/libtk_rsqref.so; None without the
    reference checkout (the library is built on the machine that generates the rsq fixtures)."""
    src = os.path.join(HERE, "tk_rsqrun.cpp")
    if not os.path.exists(REFERENCE_RSQ):
        return RSQ_LIB if os.path.exists(RSQ_LIB) else None
    os.makedirs(REF_DIR, exist_ok=True)
    deps = [src, REFERENCE_RSQ]
    if not force and os.path.exists(RSQ_LIB) and all(os.path.getmtime(RSQ_LIB) >= os.path.getmtime(d) for d in deps):
        return RSQ_LIB
    shim = os.path.join(HERE, "refshim")
    tmp = RSQ_LIB + f".tmp{os.getpid()}"
    cmd = ["g++", "-std=c++17", "-O2", "-fPIC", "-shared", "-w", "-include", os.path.join(shim, "tk_rsq_compat.h"),
           "-I", os.path.dirname(REFERENCE_RSQ), REFERENCE_RSQ, src, "-o", tmp]
    subprocess.run(cmd, check=True)
    os.replace(tmp, RSQ_LIB)
    return RSQ_LIB


if __name__ == "__main__":
    print(build_fatbin(force=True))
