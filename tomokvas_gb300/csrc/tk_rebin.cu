// tk_rebin.cu -- offset-detector (half-fan) sinogram completion and fan to
// parallel rebinning on the GPU: rsq::Half2FullFan and rsq::Half2Para /
// rsq::Fan2Para of Lukas-kV/TomoKvas (FBPG/rsq_load.cpp:327-487).
//
// A half-fan scan measures, per detector row, N angles x W columns with the
// rotation axis at column `axis_move`; the columns left of the axis are never
// measured.  Completion fills them from the conjugate rays; rebinning
// resamples the fan rays onto parallel ones.  One thread per output sample.
// The angle shift of an output column depends on the column only: the host
// forms it in FP64 as the reference does (atan / asin of the column offset)
// and passes it per column as an integer angle step plus an FP32 fraction, so
// the kernels take the two neighbouring angles exactly and interpolate in
// FP32 (the samples are FP32).
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

constexpr int kRebinMaxCols = 2048;  // output columns left of (fan) or around (parallel) the axis

// Per-column angle shifts: shift = k + frac with k an integer number of angle
// steps and frac in [0, 1) (FP32), formed on the host in FP64.
struct RebinShifts {
    short k[2][kRebinMaxCols];
    float frac[2][kRebinMaxCols];
};

// Half2FullFan (rsq_load.cpp:327-380): output row width Wc = 2W - 1 - 2am.
// Columns c >= W-1-am copy the measured half (from the axis column on);
// column c < W-1-am is the ray at detector offset t = c - (W-1-am) < 0, taken
// from the conjugate ray at offset -t and angle nf = f - (2 atan(t/D) + pi)/dfi,
// or f - (2 atan(t/D) - pi)/dfi when the first lies outside [0, N-1]; with the
// shift (2 atan(t/D) +- pi)/dfi = k + frac, nf = (f - k) - frac, so the
// two angles are f - k - 1 and f - k (one angle when frac = 0) and the weight
// of the lower is frac.  `flip` stores the angles in reverse order.
__global__ void half2fullfan_kernel(const float *__restrict__ in, float *__restrict__ out, int W, int N, int rows,
                                    int am, int flip, const __grid_constant__ RebinShifts S)
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
            // nf = (f - k) - frac; outside [0, N-1] the other conjugate (shift - 2 pi / dfi)
            int fk = f - S.k[0][c];
            float fr = S.frac[0][c];
            // nf < 0 or nf > N - 1, decided on the integer part (nf = fk - fr, fr in [0, 1))
            const bool below = fr > 0.f ? fk <= 0 : fk < 0;
            const bool above = fr > 0.f ? fk >= N : fk > N - 1;
            if (below || above) {
                fk = f - S.k[1][c];
                fr = S.frac[1][c];
            }
            const int col = c0 - c + am;  // -t + am
            // the angle past the last one wraps to the first (rsq_load.cpp:361-366); indices are
            // also wrapped and clamped for angle steps not exactly 2 pi / N
            const float A = img[(long long)wrap_angle(fk, N) * W + col];  // ceil(nf)
            if (fr == 0.f) {
                v = A;
            } else {
                const float B = img[(long long)wrap_angle(fk - 1, N) * W + col];  // floor(nf)
                v = A + (B - A) * fr;                                              // (a - nf) = frac
            }
        }
        const int fo = flip ? N - 1 - f : f;
        out[(r * N + fo) * (long long)Wc + c] = v;
    }
}

// Half2Para + Fan2Para (rsq_load.cpp:382-470): N/2 parallel angles x Wc
// columns.  Parallel column u at offset s = u - (W-1-am) samples the fan ray
// through detector column |s| + am at fan angle beta = f + asin(s/D)/dfi
// (s >= 0) or f - (asin(s/D) - pi)/dfi (s < 0), wrapped into [0, N), linearly
// interpolated between the two neighbouring fan angles.  With the shift =
// k + frac, beta = (f + k) + frac: the angles are f + k and f + k + 1 (one
// when frac = 0), the weight of the upper is frac.  As in the reference, both
// column taps use the ceiling index, so the column is never interpolated (the
// offsets are integers).
__global__ void half2para_kernel(const float *__restrict__ in, float *__restrict__ out, int W, int N, int rows,
                                 int am, const __grid_constant__ RebinShifts S)
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
        const int ui = u - (W - 1 - am);
        int fb = f + S.k[0][u];
        const float fr = S.frac[0][u];
        // beta = fb + fr, fr in [0, 1): beta < 0 iff fb < 0; beta > N - 1 decided on the integer part
        if (fb < 0) fb += N;
        if (fr > 0.f ? fb >= N - 1 : fb > N - 1) fb -= N;
        const int col = min(max((ui < 0 ? -ui : ui) + am, 0), W - 1);
        float v;
        if (fr != 0.f) {
            const float va = img[(long long)wrap_angle(fb + 1, N) * W + col];  // ceil(beta)
            const float vb = img[(long long)wrap_angle(fb, N) * W + col];      // floor(beta)
            v = va + (vb - va) * (1.f - fr);                                    // (ba - beta) = 1 - frac
        } else {
            v = img[(long long)wrap_angle(fb, N) * W + col];
        }
        out[(r * Np + f) * (long long)Wc + u] = v;
    }
}

// shift = k + frac, k = floor(shift), frac in [0, 1)
static void split_shift(double shift, short &k, float &frac)
{
    const double fl = std::floor(shift);
    k = (short)fl;
    frac = (float)(shift - fl);
    if (frac >= 1.f) {  // rounding to FP32 reached the next step
        k = (short)(k + 1);
        frac = 0.f;
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
    TK_CHECK(N <= 16384 && 2 * W - 1 - 2 * am <= kRebinMaxCols, TK_ERR_UNSUPPORTED,
             "rebin: at most 16384 angles and %d output columns", kRebinMaxCols);
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
    static thread_local RebinShifts S;
    const int c0 = W - 1 - axis_move;
    for (int c = 0; c < c0; ++c) {  // rsq_load.cpp:329-333, 352-355
        const double at = std::atan((double)(c - c0) / D);
        split_shift((2 * at + kPiD) / dfi, S.k[0][c], S.frac[0][c]);
        split_shift((2 * at - kPiD) / dfi, S.k[1][c], S.frac[1][c]);
    }
    half2fullfan_kernel<<<rebin_grid(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(
        d_in, d_out, W, N, rows, axis_move, flip ? 1 : 0, S);
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
    static thread_local RebinShifts S;
    const int Wc = 2 * W - 1 - 2 * axis_move;
    for (int u = 0; u < Wc; ++u) {  // rsq_load.cpp:409-413
        const double ui = (double)u - (double)(W - 1 - axis_move);
        const double g = ui >= 0. ? std::asin(ui / D) / dfi : -(std::asin(ui / D) - kPiD) / dfi;
        split_shift(g, S.k[0][u], S.frac[0][u]);
    }
    half2para_kernel<<<rebin_grid(total), 256, 0, static_cast<cudaStream_t>(stream)>>>(d_in, d_out, W, N, rows,
                                                                                        axis_move, S);
    count_launch();
    TK_CUDA(cudaGetLastError());
    return TK_OK;
}
