// tk_refine.cu -- data-consistency refinement of the volume with the matched
// backprojector / forward-projector pair, from checkpointed filtered
// projections.
//
// The FDK volume is x0 = B q, q = F W p: B the FP32 bilinear backprojection
// (tk_backproject with TK_F32 samples, FBPConeKernel + fQ3D of
// FBPG/kernel.cu:68-177), F W the cosine weight and ramp filter.  The
// refinement minimises the data-consistency loss
//   L(x) = || B^T x - q ||^2
// over the volume by gradient steps x <- x - alpha B (B^T x - q), with B^T the
// scatter forward projector that is B's exact transpose (tk_forward_project).
// q is the only data a step needs besides x, so it is checkpointed once after
// the filter: in FP32 samples, or where HBM is short in FP16 samples (half the
// bytes, the residual formed in FP32).  A step is three launches: B^T x into
// the FP32 residual buffer, the residual kernel (r = -alpha (B^T x - q) and
// the loss's block partials, one pass), and B r accumulated into x; a fourth
// sums the loss when it is asked for.  Sums are compensated FP32 (no FP64 on
// the device).  No counterpart in the reference, which stops at the FDK volume.
#include "tk_common.cuh"
#include "tk_internal.h"

#include <algorithm>
#include <cmath>

namespace tk {

// FP32 samples [N][H][Wp] -> FP16 samples, round to nearest.
__global__ void ckpt_to_half_kernel(const float *__restrict__ q, __half *__restrict__ out, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        out[i] = __float2half_rn(q[i]);
}

// Sums in FP32 with compensation (no FP64 on the device): each thread keeps a
// Kahan sum of its terms, each block writes its threads' total to a partial
// slot, and one block adds the partials (again compensated).  Relative error
// about 1e-6 for the sums here, far below the loss changes a step makes.
struct KahanF {
    float s = 0.f, c = 0.f;
    __device__ __forceinline__ void add(float x)
    {
        const float y = x - c;
        const float t = s + y;
        c = (t - s) - y;
        s = t;
    }
};

// Block sum (256 threads) of per-thread values into partial[blockIdx.x].
__device__ __forceinline__ void block_partial(float v, float *partial)
{
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ float wsum[8];
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) v += wsum[w];
        partial[blockIdx.x] = v;
    }
}

// r <- -alpha (r - q) over n samples; partial[block] = its part of sum (r - q)^2.
template <bool HALF>
__global__ void __launch_bounds__(256) residual_kernel(float *__restrict__ r, const void *__restrict__ ckpt,
                                                       long long n, float alpha, float *partial)
{
    KahanF acc;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        const float q = HALF ? __half2float(static_cast<const __half *>(ckpt)[i]) : static_cast<const float *>(ckpt)[i];
        const float d = r[i] - q;
        acc.add(d * d);
        r[i] = -alpha * d;
    }
    block_partial(acc.s - acc.c, partial);
}

// partial[block] = its part of sum x^2.
__global__ void __launch_bounds__(256) sumsq_kernel(const float *__restrict__ x, long long n, float *partial)
{
    KahanF acc;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        acc.add(x[i] * x[i]);
    block_partial(acc.s - acc.c, partial);
}

// *out = sum of the np partials (one block of 256 threads), widened to FP64 for the caller's loss array.
__global__ void __launch_bounds__(256) partial_sum_kernel(const float *__restrict__ partial, int np, double *out)
{
    KahanF acc;
    for (int i = threadIdx.x; i < np; i += blockDim.x) acc.add(partial[i]);
    float v = acc.s - acc.c;
    for (int o = 16; o > 0; o >>= 1) v += __shfl_xor_sync(0xffffffffu, v, o);
    __shared__ float wsum[8];
    if ((threadIdx.x & 31) == 0) wsum[threadIdx.x >> 5] = v;
    __syncthreads();
    if (threadIdx.x == 0) {
        KahanF t;
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) t.add(wsum[w]);
        *out = (double)(t.s - t.c);
    }
}

__global__ void scale_kernel(float *__restrict__ x, long long n, float s)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n; i += (long long)gridDim.x * blockDim.x)
        x[i] *= s;
}

// Deterministic pseudo-random start vector in [-1, 1) (a hash of the index): the top 24 bits of
// the hash times 2^-23, exact in FP32.
__global__ void hash_fill_kernel(float *__restrict__ x, long long n)
{
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < n;
         i += (long long)gridDim.x * blockDim.x) {
        unsigned long long h = (unsigned long long)i * 0x9E3779B97F4A7C15ull;
        h ^= h >> 31;
        h *= 0xBF58476D1CE4E5B9ull;
        h ^= h >> 29;
        x[i] = (float)(unsigned)(h >> 40) * 0x1p-23f - 1.f;
    }
}

static int grid_of(long long n)
{
    int dev = 0, sms = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev) != cudaSuccess)
        sms = 148;
    const long long want = (n + 255) / 256;
    return (int)std::max(1ll, std::min<long long>(want, (long long)sms * 8));
}

static long long residual_elems(const tk_geometry &g) { return (long long)g.N * g.H * row_pitch(g.W); }

}  // namespace tk

using namespace tk;

extern "C" size_t tk_refine_checkpoint_bytes(const tk_geometry *g, int precision)
{
    if (!g || validate_geometry(g) != TK_OK || (precision != TK_F32 && precision != TK_F16)) return 0;
    return (size_t)residual_elems(*g) * (precision == TK_F16 ? 2 : 4);
}

constexpr int kMaxPartials = 4096;  // block partial sums (grid_of never exceeds 8 blocks per SM)

// The workspace: a TK_F32 FDK workspace (its filtered-projection area is the FP32 residual),
// then kMaxPartials FP32 block partials.
static size_t partials_offset(const tk_geometry *g) { return (tk_fdk_workspace_bytes(g, TK_F32) + 255) & ~(size_t)255; }

extern "C" size_t tk_refine_workspace_bytes(const tk_geometry *g)
{
    if (!g || validate_geometry(g) != TK_OK) return 0;
    return partials_offset(g) + kMaxPartials * sizeof(float);
}

static int check_workspace(const tk_geometry *g, void *d_workspace, size_t ws_bytes)
{
    const size_t need = tk_refine_workspace_bytes(g);
    TK_CHECK(d_workspace && ws_bytes >= need, TK_ERR_INVALID, "refine: workspace of %zu B needed, %zu given", need,
             ws_bytes);
    TK_CHECK((reinterpret_cast<uintptr_t>(d_workspace) & 255) == 0, TK_ERR_INVALID,
             "refine: workspace must be 256-byte aligned");
    return TK_OK;
}

// The residual buffer: the FP32 filtered-projection area of a TK_F32 workspace
// (after its 256-byte header, which tk_refine_step_size uses for its norm).
static float *residual_of(void *d_workspace) { return reinterpret_cast<float *>(static_cast<char *>(d_workspace) + 256); }
static float *partials_of(const tk_geometry *g, void *d_workspace)
{
    return reinterpret_cast<float *>(static_cast<char *>(d_workspace) + partials_offset(g));
}

extern "C" int tk_refine_checkpoint(const tk_geometry *g, const void *d_in, int input_type, int layout,
                                    const tk_flatfield *ff, int window, void *d_ckpt, int precision,
                                    void *d_workspace, size_t workspace_bytes, void *stream)
{
    if (int rc = validate_geometry(g)) return rc;
    TK_CHECK(precision == TK_F32 || precision == TK_F16, TK_ERR_INVALID,
             "refine: the checkpoint is TK_F32 or TK_F16 samples");
    TK_CHECK(d_in && d_ckpt, TK_ERR_INVALID, "refine: null device pointer");
    if (int rc = check_workspace(g, d_workspace, workspace_bytes)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    // q = F W p in FP32 samples [N][H][Wp] (the FFT form: the filter of the FP32 FDK)
    float *q = precision == TK_F32 ? static_cast<float *>(d_ckpt) : residual_of(d_workspace);
    if (int rc = launch_filter(*g, d_in, input_type, layout, ff, window, q, TK_F32, nullptr, st, 0, 0, TK_FILTER_FFT))
        return rc;
    if (precision == TK_F16) {
        const long long n = residual_elems(*g);
        ckpt_to_half_kernel<<<grid_of(n), 256, 0, st>>>(q, static_cast<__half *>(d_ckpt), n);
        TK_CUDA(cudaGetLastError());
        count_launch();
    }
    return TK_OK;
}

extern "C" int tk_refine_volume(const tk_geometry *g, const void *d_ckpt, int precision, float alpha, int steps,
                                float *d_vol, double *d_loss, void *d_workspace, size_t workspace_bytes,
                                void *stream)
{
    if (int rc = validate_geometry(g)) return rc;
    TK_CHECK(precision == TK_F32 || precision == TK_F16, TK_ERR_INVALID,
             "refine: the checkpoint is TK_F32 or TK_F16 samples");
    TK_CHECK(d_ckpt && d_vol, TK_ERR_INVALID, "refine: null device pointer");
    TK_CHECK(steps >= 0, TK_ERR_INVALID, "refine: steps < 0");
    TK_CHECK(std::isfinite(alpha) && alpha > 0.f, TK_ERR_INVALID, "refine: step size must be positive");
    if (int rc = check_workspace(g, d_workspace, workspace_bytes)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *r = residual_of(d_workspace), *partials = partials_of(g, d_workspace);
    const long long n = residual_elems(*g);
    const int grid = grid_of(n);
    TK_CHECK(grid <= kMaxPartials, TK_ERR_UNSUPPORTED, "refine: %d blocks exceed the partial sums", grid);
    const float zoff = tk_default_zoff(g);
    for (int k = 0; k < steps; ++k) {
        // B^T x, then r = -alpha (B^T x - q) with the loss's block partials, then x += B r
        if (int rc = launch_forward_project(*g, d_vol, g->Z, zoff, r, 0, st)) return rc;
        if (precision == TK_F16)
            residual_kernel<true><<<grid, 256, 0, st>>>(r, d_ckpt, n, alpha, partials);
        else
            residual_kernel<false><<<grid, 256, 0, st>>>(r, d_ckpt, n, alpha, partials);
        TK_CUDA(cudaGetLastError());
        count_launch();
        if (d_loss) {
            partial_sum_kernel<<<1, 256, 0, st>>>(partials, grid, d_loss + k);
            TK_CUDA(cudaGetLastError());
            count_launch();
        }
        if (int rc = launch_backproject(*g, r, TK_F32, nullptr, g->Z, zoff, d_vol, 1, st)) return rc;
    }
    return TK_OK;
}

extern "C" int tk_refine_step_size(const tk_geometry *g, int iters, float *d_vol_tmp, void *d_workspace,
                                   size_t workspace_bytes, float *alpha_out, void *stream)
{
    if (int rc = validate_geometry(g)) return rc;
    TK_CHECK(d_vol_tmp && alpha_out, TK_ERR_INVALID, "refine: null pointer");
    TK_CHECK(iters >= 1, TK_ERR_INVALID, "refine: iters < 1");
    if (int rc = check_workspace(g, d_workspace, workspace_bytes)) return rc;
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *r = residual_of(d_workspace), *partials = partials_of(g, d_workspace);
    double *acc = reinterpret_cast<double *>(d_workspace);  // the workspace header holds the norm
    const long long nv = (long long)g->X * g->Y * g->Z;
    const int grid = grid_of(nv);
    TK_CHECK(grid <= kMaxPartials, TK_ERR_UNSUPPORTED, "refine: %d blocks exceed the partial sums", grid);
    const float zoff = tk_default_zoff(g);
    // power iteration on B B^T from a fixed pseudo-random volume: lambda = ||B B^T x|| for ||x|| = 1
    hash_fill_kernel<<<grid_of(nv), 256, 0, st>>>(d_vol_tmp, nv);
    count_launch();
    double lambda = 0.0, norm = 0.0;
    for (int it = -1; it < iters; ++it) {
        if (it >= 0) {
            if (int rc = launch_forward_project(*g, d_vol_tmp, g->Z, zoff, r, 0, st)) return rc;
            if (int rc = launch_backproject(*g, r, TK_F32, nullptr, g->Z, zoff, d_vol_tmp, 0, st)) return rc;
        }
        sumsq_kernel<<<grid, 256, 0, st>>>(d_vol_tmp, nv, partials);
        partial_sum_kernel<<<1, 256, 0, st>>>(partials, grid, acc);
        TK_CUDA(cudaGetLastError());
        count_launch(2);
        TK_CUDA(cudaMemcpyAsync(&norm, acc, sizeof(double), cudaMemcpyDeviceToHost, st));
        TK_CUDA(cudaStreamSynchronize(st));
        norm = std::sqrt(norm);
        TK_CHECK(norm > 0.0 && std::isfinite(norm), TK_ERR_DEVICE, "refine: power iteration lost its vector");
        if (it >= 0) lambda = norm;  // the previous vector had unit norm
        scale_kernel<<<grid_of(nv), 256, 0, st>>>(d_vol_tmp, nv, (float)(1.0 / norm));
        count_launch();
    }
    TK_CUDA(cudaStreamSynchronize(st));
    TK_CHECK(lambda > 0.0, TK_ERR_DEVICE, "refine: B B^T has no positive eigenvalue estimate");
    *alpha_out = (float)(1.0 / lambda);
    return TK_OK;
}
