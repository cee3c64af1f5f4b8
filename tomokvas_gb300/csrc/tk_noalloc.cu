// tk_noalloc.cu -- whole-FDK entry point that allocates no memory.
//
// Some callers cannot call cudaMalloc: an acquisition or reconstruction
// service that reserves a fixed device-memory budget at start-up and may not
// grow it afterwards, or code that runs inside a callback or a timing-critical
// loop where cudaMalloc's implicit device synchronisation and its possible
// failure are not acceptable.  tk_fdk_device_noalloc serves them: it runs
// the same filter and backprojection as tk_fdk_device, with the workspace
// (the filtered projections and their scale word) in a file-scope device
// array of kNoAllocScratchBytes instead of caller-provided memory.
//
// The array exists once per GPU on which this module is loaded and stays
// allocated until the process exits.  Every call shares it and it keeps the
// previous call's contents; the filter rewrites everything the
// backprojection reads, including the scale word, so nothing needs clearing.
// Calls whose work overlaps on the GPU (other streams, other host threads)
// race on the array: serialise them.
#include "tk_common.cuh"
#include "tk_internal.h"

#include <mutex>

namespace tk {

constexpr size_t kNoAllocScratchBytes = 64ull << 20;  // 64 MiB

static __device__ __align__(256) unsigned char g_noalloc_scratch[kNoAllocScratchBytes];

// Device address of the array for the current device, looked up once per
// device with that device current.  The first call on a device does this
// set-up, so it should be made before any stream capture.
static int noalloc_scratch(void **out)
{
    static std::mutex mu;
    static void *addr[64] = {};
    int dev = 0;
    TK_CUDA(cudaGetDevice(&dev));
    TK_CHECK(dev >= 0 && dev < 64, TK_ERR_UNSUPPORTED, "device ordinal %d beyond 63", dev);
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        const cudaError_t e = cudaGetSymbolAddress(&p, g_noalloc_scratch);
        if (e != cudaSuccess) return cuda_fail(e, "cudaGetSymbolAddress(no-alloc scratch)");
        addr[dev] = p;
    }
    *out = addr[dev];
    return TK_OK;
}

}  // namespace tk

extern "C" int tk_fdk_device_noalloc(const tk_geometry *g, const void *d_in, int input_type, int layout,
                                     const tk_flatfield *ff, int window, int precision, float *d_vol, void *stream)
{
    if (int rc = tk::validate_geometry(g)) return rc;
    TK_CHECK(tk::valid_precision(precision), TK_ERR_INVALID, "bad precision %d", precision);
    const size_t need = tk_fdk_workspace_bytes(g, precision);
    TK_CHECK(need <= tk::kNoAllocScratchBytes, TK_ERR_UNSUPPORTED,
             "no-alloc FDK: this problem needs %zu B of workspace, more than the %zu B static scratch; "
             "use tk_fdk_device with a caller-provided workspace",
             need, tk::kNoAllocScratchBytes);
    void *scratch = nullptr;
    if (int rc = tk::noalloc_scratch(&scratch)) return rc;
    return tk_fdk_device(g, d_in, input_type, layout, ff, window, precision, scratch, tk::kNoAllocScratchBytes, d_vol,
                         stream);
}
