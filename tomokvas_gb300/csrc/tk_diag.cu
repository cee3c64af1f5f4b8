// tk_diag.cu -- measurement helpers of the library: a count of the kernels
// it has launched, and a live measurement of the GPU's FP32 FMA rate (the
// denominator of the backprojection's roofline, which is bound by the FP32
// pipe rather than by HBM or the tensor cores).
#include "tk_common.cuh"
#include "tk_internal.h"

#include <atomic>

namespace tk {

static std::atomic<unsigned long long> g_launches{0};

void count_launch(unsigned n) { g_launches.fetch_add(n, std::memory_order_relaxed); }

// Eight independent FMA chains per thread, a fixed trip count; one store per
// thread keeps the work alive.
__global__ void __launch_bounds__(256) fma_rate_kernel(float *out, float s, int iters)
{
    float a[8];
#pragma unroll
    for (int i = 0; i < 8; ++i) a[i] = threadIdx.x * 1e-3f + i;
    for (int it = 0; it < iters; ++it) {
#pragma unroll
        for (int i = 0; i < 8; ++i) a[i] = fmaf(a[i], s, 0.5f);
    }
    float r = 0.f;
#pragma unroll
    for (int i = 0; i < 8; ++i) r += a[i];
    out[blockIdx.x * blockDim.x + threadIdx.x] = r;
}

// A wait that nothing completes: one thread arms an mbarrier for 1024 bytes of
// asynchronous copies and issues none, then waits with the library's bounded
// wait; when the limit runs out it reports ERR_WAIT_TIMEOUT in the error word
// and the CTA returns (no copy is in flight), as every kernel of the library
// does when a stage never lands.
__global__ void wait_timeout_kernel(unsigned *err, unsigned long long limit_ns)
{
    __shared__ uint64_t bar;
    if (threadIdx.x == 0) {
        mbar_init(&bar, 1);
        fence_mbar_init();
        mbar_arrive_expect_tx(&bar, 1024);
    }
    __syncthreads();
    if (threadIdx.x == 0 && !mbar_wait_bounded(&bar, 0, limit_ns)) atomicOr(err, ERR_WAIT_TIMEOUT);
}

}  // namespace tk

using namespace tk;

extern "C" int tk_diag_wait_timeout(double limit_ms, void *stream)
{
    TK_CHECK(limit_ms > 0 && limit_ms <= 1000, TK_ERR_INVALID, "tk_diag_wait_timeout: limit outside (0, 1000] ms");
    unsigned *err = device_error_word();
    TK_CHECK(err, TK_ERR_CUDA, "device error word unavailable");
    wait_timeout_kernel<<<1, 32, 0, static_cast<cudaStream_t>(stream)>>>(err, (unsigned long long)(limit_ms * 1e6));
    TK_CUDA(cudaGetLastError());
    count_launch();
    return TK_OK;
}

extern "C" unsigned long long tk_kernel_launches(void) { return g_launches.load(std::memory_order_relaxed); }

extern "C" int tk_measure_fp32_fma_rate(double *tflops_out)
{
    TK_CHECK(tflops_out, TK_ERR_INVALID, "tk_measure_fp32_fma_rate: null output");
    int dev = 0, sms = 0;
    TK_CUDA(cudaGetDevice(&dev));
    TK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const int blocks = sms * 8, threads = 256, iters = 4096;
    float *out = nullptr;
    TK_CUDA(cudaMalloc(&out, sizeof(float) * (size_t)blocks * threads));
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    cudaEventCreate(&e0);
    cudaEventCreate(&e1);
    float best = 3.0e38f;
    int rc = TK_OK;
    for (int rep = 0; rep < 3 && rc == TK_OK; ++rep) {
        cudaEventRecord(e0);
        fma_rate_kernel<<<blocks, threads>>>(out, 0.999f, iters);
        cudaEventRecord(e1);
        if (cudaEventSynchronize(e1) != cudaSuccess) rc = cuda_fail(cudaGetLastError(), "fma rate kernel");
        float ms = 0.f;
        if (rc == TK_OK) cudaEventElapsedTime(&ms, e0, e1);
        if (rep > 0 && ms < best) best = ms;  // the first run is a warm-up
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(out);
    if (rc) return rc;
    *tflops_out = 2.0 * blocks * threads * (double)iters * 8 / (best * 1e-3) / 1e12;
    return TK_OK;
}
