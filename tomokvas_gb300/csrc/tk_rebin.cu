// tk_rebin.cu -- offset-detector (half-fan) sinogram completion and fan to
// parallel rebinning on the GPU: rsq::Half2FullFan and rsq::Half2Para /
// rsq::Fan2Para of Lukas-kV/TomoKvas (FBPG/rsq_load.cpp:327-487).
//
// A half-fan scan measures, per detector row, N angles x W columns with the
// rotation axis at column `axis_move`; the columns left of the axis are never
// measured.  Completion fills them from the conjugate rays; rebinning
// resamples the fan rays onto parallel ones.  One thread per output sample;
// the angle arithmetic is FP64 as in the reference (it runs once per output,
// not per voxel), the samples are FP32.
#include "tk_common.cuh"
#include "tk_internal.h"

#include <cmath>

namespace tk {

constexpr double kPiD = 3.14159265358979323846;

// Angle index modulo N, clamped into [0, N-1].
__device__ __forceinline__ int wrap_angle(int a, int N)
{
    if (a > N - 1) a -= N;
    if (a < 0) a += N;
    return min(max(a, 0), N - 1);
}

// Half2FullFan (rsq_load.cpp:327-380): output row width Wc = 2W - 1 - 2am.
// Columns c >= W-1-am copy the measured half (from the axis column on);
// column c < W-1-am is the ray at detector offset t = c - (W-1-am) < 0, taken
// from the conjugate ray at offset -t and angle f - (2 atan(t/D) + pi)/dfi
// (+ N when that is negative), linearly interpolated between its two angles.
// `flip` stores the angles in reverse order.
__global__ void half2fullfan_kernel(const float *__restrict__ in, float *__restrict__ out, int W, int N, int rows,
                                    int am, double D, double dfi, int flip)
{
    const int Wc = 2 * W - 1 - 2 * am;
    const long long total = (long long)rows * N * Wc;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int c = (int)(i % Wc);
        const long long rf = i / Wc;
        const int f = (int)(rf % N);
        const long long r = rf / N;
        const float *img = in + r * (long long)N * W;
        const int c0 = W - 1 - am;  // output column of the axis
        float v;
        if (c >= c0) {
            v = img[(long long)f * W + (c - c0) + am];
        } else {
            const int t = c - c0;  // < 0
            const double at = atan((double)t / D);
            const double fi = (double)f * dfi;
            double nf = (fi - 2 * at - kPiD) / dfi;
            if (nf > (N - 1) || nf < 0) nf = (fi - 2 * at + kPiD) / dfi;
            const int a = (int)ceil(nf), b = (int)floor(nf);
            const int col = -t + am;
            // the angle past the last one wraps to the first (rsq_load.cpp:361-366); indices are
            // also wrapped and clamped for angle steps not exactly 2 pi / N
            const float A = img[(long long)wrap_angle(a, N) * W + col];
            const float B = img[(long long)wrap_angle(b, N) * W + col];
            v = (a != b) ? (float)((double)A + ((double)B - (double)A) * ((double)a - nf)) : A;
        }
        const int fo = flip ? N - 1 - f : f;
        out[(r * N + fo) * (long long)Wc + c] = v;
    }
}

// Half2Para + Fan2Para (rsq_load.cpp:382-470): N/2 parallel angles x Wc
// columns.  Parallel column u at offset s = u - (W-1-am) samples the fan ray
// through detector column |s| + am at fan angle f + asin(s/D)/dfi (s >= 0) or
// f - (asin(s/D) - pi)/dfi (s < 0), wrapped into [0, N), linearly
// interpolated between the two neighbouring fan angles.  As in the
// reference, both column taps use the ceiling index, so the column is never
// interpolated (the offsets are integers).
__global__ void half2para_kernel(const float *__restrict__ in, float *__restrict__ out, int W, int N, int rows,
                                 int am, double D, double dfi)
{
    const int Wc = 2 * W - 1 - 2 * am, Np = N / 2;
    const long long total = (long long)rows * Np * Wc;
    for (long long i = blockIdx.x * (long long)blockDim.x + threadIdx.x; i < total;
         i += (long long)gridDim.x * blockDim.x) {
        const int u = (int)(i % Wc);
        const long long rf = i / Wc;
        const int f = (int)(rf % Np);
        const long long r = rf / Np;
        const float *img = in + r * (long long)N * W;
        const double ui = (double)u - (double)(W - 1 - am);
        double beta = ui >= 0. ? f + asin(ui / D) / dfi : f - (asin(ui / D) - kPiD) / dfi;
        double s = ui;
        if (beta < 0.) beta += N;
        if (beta > N - 1) beta -= N;
        if (ui < 0.) s = -s;
        const int ba = (int)ceil(beta), bb = (int)floor(beta);
        const int col = min(max((int)ceil(s) + am, 0), W - 1);
        float v;
        if (ba != bb) {
            const float va = img[(long long)wrap_angle(ba, N) * W + col];
            const float vb = img[(long long)wrap_angle(bb, N) * W + col];
            v = (float)((double)va + ((double)vb - (double)va) * ((double)ba - beta));
        } else {
            v = img[(long long)wrap_angle(ba, N) * W + col];
        }
        out[(r * Np + f) * (long long)Wc + u] = v;
    }
}

static int rebin_check(const float *d_in, float *d_out, int W, int N, int rows, int am, double D, double dfi)
{
    TK_CHECK(d_in && d_out, TK_ERR_INVALID, "rebin: null device pointer");
    TK_CHECK(W > 1 && N > 1 && rows > 0, TK_ERR_INVALID, "rebin: bad sizes %d x %d x %d", W, N, rows);
    TK_CHECK(am >= 0 && am < W - 1, TK_ERR_INVALID, "rebin: axis_move %d outside [0, W-1)", am);
    TK_CHECK(std::isfinite(D) && D > W && std::isfinite(dfi) && dfi > 0, TK_ERR_INVALID,
             "rebin: need D > W (pixels) and dfi > 0");
    TK_CHECK(std::fabs(dfi * N - 2 * kPiD) < 1e-3, TK_ERR_UNSUPPORTED, "rebin: needs a full 360-degree scan");
    return TK_OK;
}

static dim3 rebin_grid(long long total)
{
    int dev = 0, sms = 1;
    cudaGetDevice(&dev);
    cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev);
    const long long blocks = (total + 255) / 256;
    return dim3((unsigned)std::min<long long>(blocks, (long long)sms * 16));
}

}  // namespace tk

using namespace tk;

extern "C" int tk_half_to_full_fan(const float *d_in, int W, int N, int rows, int axis_move, double D, double dfi,
                                   int flip, float *d_out, void *stream)
{
    if (int rc = rebin_check(d_in, d_out, W, N, rows, axis_move, D, dfi)) return rc;
    const long long total = (long long)rows * N * (2 * W - 1 - 2 * axis_move);
    half2fullfan_kernel<<<rebin_grid(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        d_in, d_out, W, N, rows, axis_move, D, dfi, flip ? 1 : 0);
    count_launch();
    TK_CUDA(cudaGetLastError());
    return TK_OK;
}

extern "C" int tk_half_to_parallel(const float *d_in, int W, int N, int rows, int axis_move, double D, double dfi,
                                   float *d_out, void *stream)
{
    if (int rc = rebin_check(d_in, d_out, W, N, rows, axis_move, D, dfi)) return rc;
    TK_CHECK(N % 2 == 0, TK_ERR_INVALID, "rebin: parallel rebinning needs an even number of angles");
    const long long total = (long long)rows * (N / 2) * (2 * W - 1 - 2 * axis_move);
    half2para_kernel<<<rebin_grid(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(d_in, d_out, W, N, rows,
                                                                                        axis_move, D, dfi);
    count_launch();
    TK_CUDA(cudaGetLastError());
    return TK_OK;
}
