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
"""
import os
import subprocess

HERE = os.path.dirname(os.path.abspath(__file__))
REF_DIR = os.path.join(HERE, "_ref")
FATBIN = os.path.join(REF_DIR, "tk_ref_kernels.fatbin")
LOADER = os.path.join(REF_DIR, "libtk_ref.so")
REFERENCE_KERNEL = "/root/reference/FBPG/kernel.cu"
CUDA = "/usr/local/cuda"


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


if __name__ == "__main__":
    print(build_fatbin(force=True))
