// tk_filter.cu -- fused preprocessing + ramp filter for GB300 (sm_103a).
//
// Replaces three stages of the reference FDK (Lukas-kV/TomoKvas):
//   * raw uint16 -> line integral, rsq::FlatFieldCorrection (FBPG/rsq_load.cpp:299-325);
//   * cosine pre-weight, RB_comma3DKernel (FBPG/kernel.cu:179-201);
//   * row-wise ramp filter, fConvolution (FBPG/kernel.cu:557-781): per detector
//     row, zero-pad to p = 2*nextpow2(W), R2C, multiply by tau*|R2C(h)|, C2R
//     unnormalised.
//
// GB300 design: one pass over HBM.  Each CTA streams pairs of detector rows
// straight from the raw input, applies log + cosine weight while loading,
// packs the two real rows as one complex signal z = a + i b, and runs a
// radix-4/2 Stockham FFT in shared memory.  Because the filter spectrum is
// real and even, IFFT(FFT(z) * Hf) = (a*k) + i (b*k), so one forward and one
// inverse complex FFT filter two rows.  The inverse is computed as
// conj(FFT(conj(Z) * Hf)).  Results are written once, projection-major, in
// FP32/FP16/BF16.  No cuFFT, no staging copies, no per-row plans.
#include "tk_common.cuh"
#include "tk_filter_core.cuh"
#include "tk_internal.h"

#include <cmath>
#include <cstring>
#include <map>
#include <mutex>
#include <tuple>
#include <vector>

namespace tk {

constexpr int kMaxHf = 4097;  // p/2 + 1 for p <= 8192
constexpr int kFiltThreads = 256;
constexpr float kScaleTarget = 16384.f;  // bound of |stored value| for 16-bit storage

// ---------------------------------------------------------------------------
// Mixed-radix Stockham FFT in shared memory.
//
// A length p = 2^lg transform runs as radix-16 passes and one final radix
// 8/4/2 pass (p = 2048: 16, 16, 8).  Pass m with span Ns and radix R maps
// butterfly j (k = j mod Ns) as
//   v[r] = x[j + r p/R] * w^(r k p/(R Ns)),  y[(j-k) R + k + s Ns] = DFT_R(v)[s],
// one butterfly per thread, the R points in registers.  Buffers are padded by
// one element per 16 (pidx), which makes every pass's loads and stores
// conflict-free; twiddles come from per-pass tables laid out [k][r] (one
// thread reads R-1 consecutive entries).
struct FFTPlan {
    int npass;
    int R[5], Ns[5], off[5];  // radix, span and twiddle-table offset of each pass
    int tw_total;             // twiddle entries of all passes
};

__host__ __device__ inline FFTPlan fft_plan(int lg)
{
    FFTPlan pl{};
    int Ns = 1, rem = lg, off = 0;
    while (rem > 0) {
        const int b = rem >= 4 ? 4 : rem;
        const int R = 1 << b;
        pl.R[pl.npass] = R;
        pl.Ns[pl.npass] = Ns;
        pl.off[pl.npass] = off;
        if (Ns > 1) off += Ns * (R - 1);
        Ns *= R;
        rem -= b;
        ++pl.npass;
    }
    pl.tw_total = off;
    return pl;
}

struct FiltParams {
    LoadParams L;
    void *out;
    const float *q_scale;  // device storage scale (16-bit) or null (= 1)
    long long nrows, npairs;
    int Wp, p, lg, precision;
    int rc, nchunks;        // coefficient image: rows per work unit, units per projection
    long long nunits;
    int fgrp, fstride;      // coefficient image, frames in groups (> 0): frame f is f/fgrp*fstride + f%fgrp
    int out_layout;         // raw output: TK_LAYOUT_PROJECTION [N][H][Wp] or TK_LAYOUT_SINOGRAM [H][N][Wp]
    int weight_out;         // multiply the output by the cosine weight (the filter's transpose)
    FFTPlan plan;           // passes of the length-p transform (fft_plan(lg))
    float Hf[kMaxHf];  // tau * |R2C_p(h)| * window, k = 0..p/2
};

// Raw samples x0 .. x0+NV-1 of the row at element offset off; samples at or
// past W read as 0.  With L.vec the run is read with 16-byte loads (the run
// starts on a 16-byte boundary: x0 is a multiple of NV, NV * element size is
// a multiple of 16, rows start aligned and the row pitch covers every chunk
// that starts below W).
template <int NV>
__device__ __forceinline__ void load_run(const LoadParams &L, long long off, int x0, bool valid, float (&v)[NV])
{
#pragma unroll
    for (int j = 0; j < NV; ++j) v[j] = 0.f;
    if (!valid) return;
    if constexpr (NV % 8 == 0) {
        if (L.vec && L.input_type == TK_INPUT_U16) {
            const uint4 *src = reinterpret_cast<const uint4 *>(static_cast<const uint16_t *>(L.in) + off + x0);
#pragma unroll
            for (int k = 0; k < NV / 8; ++k) {
                if (x0 + 8 * k < L.W) {
                    const uint4 q = __ldg(src + k);
                    const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
                    for (int e = 0; e < 4; ++e) {
                        v[8 * k + 2 * e] = (float)(w[e] & 0xffffu);
                        v[8 * k + 2 * e + 1] = (float)(w[e] >> 16);
                    }
                }
            }
#pragma unroll
            for (int j = 0; j < NV; ++j)
                if (x0 + j >= L.W) v[j] = 0.f;
            return;
        }
    }
    if constexpr (NV % 4 == 0) {
        if (L.vec && L.input_type == TK_INPUT_F32) {
            const float4 *src = reinterpret_cast<const float4 *>(static_cast<const float *>(L.in) + off + x0);
#pragma unroll
            for (int k = 0; k < NV / 4; ++k) {
                if (x0 + 4 * k < L.W) {
                    const float4 q = __ldg(src + k);
                    v[4 * k] = q.x;
                    v[4 * k + 1] = q.y;
                    v[4 * k + 2] = q.z;
                    v[4 * k + 3] = q.w;
                }
            }
#pragma unroll
            for (int j = 0; j < NV; ++j)
                if (x0 + j >= L.W) v[j] = 0.f;
            return;
        }
    }
#pragma unroll
    for (int j = 0; j < NV; ++j)
        if (x0 + j < L.W) v[j] = load_raw(L, off, x0 + j);
}

__device__ __forceinline__ float2 cmul(float2 a, float2 b)
{
    return make_float2(a.x * b.x - a.y * b.y, a.x * b.y + a.y * b.x);
}
__device__ __forceinline__ float2 cadd(float2 a, float2 b) { return make_float2(a.x + b.x, a.y + b.y); }
__device__ __forceinline__ float2 csub(float2 a, float2 b) { return make_float2(a.x - b.x, a.y - b.y); }

// Padded index of element i of a transform buffer.
__host__ __device__ __forceinline__ int pidx(int i) { return i + (i >> 4); }
__host__ __device__ __forceinline__ int padded_len(int p) { return p + (p >> 4); }

// Twiddle tables of every pass: entry (k, r) of pass m is w^(r k p/(R Ns)) =
// exp(-2 pi i r k / (R Ns)), r = 1..R-1, k < Ns.  All threads of the CTA.
__device__ __forceinline__ void fill_twiddles(float2 *twp, const FFTPlan &pl)
{
#pragma unroll
    for (int m = 0; m < 4; ++m) {
        if (m >= pl.npass) break;
        const int R = pl.R[m], Ns = pl.Ns[m];
        if (Ns == 1) continue;
        for (int i = threadIdx.x; i < Ns * (R - 1); i += blockDim.x) {
            const int k = i / (R - 1), r = i - k * (R - 1) + 1;
            float sn, cs;
            sincospif(-2.0f * (float)(r * k) / (float)(R * Ns), &sn, &cs);  // exact argument: R Ns is 2^n
            twp[pl.off[m] + i] = make_float2(cs, sn);
        }
    }
}

// Forward DFTs of 2, 4, 8 and 16 points in registers (natural order).
__device__ __forceinline__ void dft2(float2 &a, float2 &b)
{
    const float2 t = a;
    a = cadd(t, b);
    b = csub(t, b);
}
__device__ __forceinline__ void dft4(float2 &x0, float2 &x1, float2 &x2, float2 &x3)
{
    const float2 a = cadd(x0, x2), b = csub(x0, x2), c = cadd(x1, x3), d = csub(x1, x3);
    x0 = cadd(a, c);
    x2 = csub(a, c);
    x1 = make_float2(b.x + d.y, b.y - d.x);  // b - i d
    x3 = make_float2(b.x - d.y, b.y + d.x);  // b + i d
}
constexpr float kR2 = 0.70710678118654752440f;  // cos(pi/4)
constexpr float kC8 = 0.92387953251128675613f;  // cos(pi/8)
constexpr float kS8 = 0.38268343236508977173f;  // sin(pi/8)

template <int R> __device__ __forceinline__ void dft(float2 (&v)[R]);
template <> __device__ __forceinline__ void dft<2>(float2 (&v)[2]) { dft2(v[0], v[1]); }
template <> __device__ __forceinline__ void dft<4>(float2 (&v)[4]) { dft4(v[0], v[1], v[2], v[3]); }
// 8 = 2 x 4: X[k + 4h] = E0[k] + (-1)^h W8^k E1[k], E_e = DFT4(x[e], x[e+2], x[e+4], x[e+6]).
template <> __device__ __forceinline__ void dft<8>(float2 (&v)[8])
{
    dft4(v[0], v[2], v[4], v[6]);
    dft4(v[1], v[3], v[5], v[7]);
    const float2 t1 = make_float2(kR2 * (v[3].x + v[3].y), kR2 * (v[3].y - v[3].x));   // W8^1 = (r, -r)
    const float2 t2 = make_float2(v[5].y, -v[5].x);                                     // W8^2 = -i
    const float2 t3 = make_float2(kR2 * (v[7].y - v[7].x), -kR2 * (v[7].x + v[7].y));  // W8^3 = (-r, -r)
    const float2 e0 = v[0], e1 = v[2], e2 = v[4], e3 = v[6];
    v[0] = cadd(e0, v[1]);
    v[4] = csub(e0, v[1]);
    v[1] = cadd(e1, t1);
    v[5] = csub(e1, t1);
    v[2] = cadd(e2, t2);
    v[6] = csub(e2, t2);
    v[3] = cadd(e3, t3);
    v[7] = csub(e3, t3);
}
// 16 = 4 x 4: E_e = DFT4(x[e], x[e+4], x[e+8], x[e+12]); T_e[k] = W16^(e k) E_e[k];
// X[k + 4h] = DFT4_h(T_0[k], T_1[k], T_2[k], T_3[k]).
template <> __device__ __forceinline__ void dft<16>(float2 (&v)[16])
{
#pragma unroll
    for (int e = 0; e < 4; ++e) dft4(v[e], v[e + 4], v[e + 8], v[e + 12]);
    // E_e[k] sits in v[e + 4k]; apply W16^(e k)
    const float2 w1 = make_float2(kC8, -kS8), w2 = make_float2(kR2, -kR2), w3 = make_float2(kS8, -kC8);
    const float2 w6 = make_float2(-kR2, -kR2), w9 = make_float2(-kC8, kS8);
    v[5] = cmul(v[5], w1);                          // e=1,k=1
    v[9] = cmul(v[9], w2);                          // e=1,k=2
    v[13] = cmul(v[13], w3);                        // e=1,k=3
    v[6] = cmul(v[6], w2);                          // e=2,k=1
    v[10] = make_float2(v[10].y, -v[10].x);         // e=2,k=2: W16^4 = -i
    v[14] = cmul(v[14], w6);                        // e=2,k=3
    v[7] = cmul(v[7], w3);                          // e=3,k=1
    v[11] = cmul(v[11], w6);                        // e=3,k=2
    v[15] = cmul(v[15], w9);                        // e=3,k=3
    float2 o[16];
#pragma unroll
    for (int k = 0; k < 4; ++k) {
        float2 a = v[4 * k], b = v[4 * k + 1], c = v[4 * k + 2], d = v[4 * k + 3];
        dft4(a, b, c, d);
        o[k] = a;
        o[k + 4] = b;
        o[k + 8] = c;
        o[k + 12] = d;
    }
#pragma unroll
    for (int i = 0; i < 16; ++i) v[i] = o[i];
}

// Threads per transform (one radix-16 butterfly each); compile-time form.
__host__ __device__ constexpr int fft_threads_c(int p)
{
    return ((p >> 4) > 32 ? (p >> 4) : 32) < kFiltThreads ? ((p >> 4) > 32 ? (p >> 4) : 32) : kFiltThreads;
}

// Compile-time length: pass m of a length-2^LG transform has radix 16 except
// possibly the last (fft_plan), span Ns = 16^m and its twiddle table at
// offset 16^m - 16 (m >= 1).  With every size a constant, the padded
// addresses of the loads and stores fold into immediates and the butterfly
// loops unroll.
template <int R, int P, int NS>
__device__ __forceinline__ void fft_pass_c(const float2 *__restrict__ x, float2 *__restrict__ y,
                                           const float2 *__restrict__ tw, int t)
{
    constexpr int Q = P / R;
    constexpr int TPF = fft_threads_c(P);
    constexpr int ITER = (Q + TPF - 1) / TPF;
#pragma unroll
    for (int i = 0; i < ITER; ++i) {
        const int j = t + i * TPF;
        if ((Q % TPF) != 0 && j >= Q) break;
        const int k = j & (NS - 1);
        float2 v[R];
        if constexpr (Q % 16 == 0) {  // pidx(j + r Q) = pidx(j) + r (Q + Q/16)
            const float2 *xs = x + pidx(j);
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = xs[r * (Q + Q / 16)];
        } else {
#pragma unroll
            for (int r = 0; r < R; ++r) v[r] = x[pidx(j + r * Q)];
        }
        if constexpr (NS > 1) {
            const float2 *w = tw + k * (R - 1) - 1;
#pragma unroll
            for (int r = 1; r < R; ++r) v[r] = cmul(v[r], w[r]);
        }
        dft<R>(v);
        const int o = (j - k) * R + k;
        if constexpr (NS % 16 == 0) {
            float2 *ys = y + pidx(o);
#pragma unroll
            for (int s2 = 0; s2 < R; ++s2) ys[s2 * (NS + NS / 16)] = v[s2];
        } else if constexpr (NS == 1 && R == 16) {  // o is a multiple of 16: o + s stays in one padding group
            float2 *ys = y + pidx(o);
#pragma unroll
            for (int s2 = 0; s2 < R; ++s2) ys[s2] = v[s2];
        } else {
#pragma unroll
            for (int s2 = 0; s2 < R; ++s2) y[pidx(o + s2 * NS)] = v[s2];
        }
    }
}

// Barrier of the TPF threads of transform group grp (named barrier 1 + grp):
// the groups of a CTA share only read-only tables, so none waits on another.
template <int TPF>
__device__ __forceinline__ void group_sync(int grp)
{
    asm volatile("bar.sync %0, %1;" ::"r"(grp + 1), "n"(TPF) : "memory");
}

template <int LG, int M>
__device__ __forceinline__ void fft_passes_c(float2 *&a, float2 *&b, const float2 *twp, int t, int grp)
{
    if constexpr (LG - 4 * M > 0) {
        constexpr int rem = LG - 4 * M;
        constexpr int R = rem >= 4 ? 16 : (1 << rem);
        constexpr int NS = 1 << (4 * M);
        constexpr int OFF = M >= 1 ? (1 << (4 * M)) - 16 : 0;
        fft_pass_c<R, (1 << LG), NS>(a, b, twp + OFF, t);
        group_sync<fft_threads_c(1 << LG)>(grp);
        float2 *s2 = a;
        a = b;
        b = s2;
        fft_passes_c<LG, M + 1>(a, b, twp, t, grp);
    }
}

// Forward FFT of length 2^LG (padded buffers); ping-pongs between a and b and
// returns the buffer holding the result.  Every thread of the transform group
// calls it (group barriers inside).
template <int LG>
__device__ __forceinline__ float2 *fft_forward_c(float2 *a, float2 *b, const float2 *twp, int t, int grp)
{
    fft_passes_c<LG, 0>(a, b, twp, t, grp);
    return a;
}

// Threads per transform (one radix-16 butterfly each) and groups per CTA.
__host__ __device__ __forceinline__ int fft_threads(int p)
{
    const int t = (p >> 4) > 32 ? (p >> 4) : 32;
    return t < kFiltThreads ? t : kFiltThreads;
}

// Shared-memory layout of the filter kernels: twiddle tables, the spectrum
// Hf (p/2+1 floats), then per group two padded transform buffers.
struct FiltSmem {
    int tw_total, hf_floats, group_bytes, groups;
    __host__ __device__ size_t bytes() const
    {
        return (size_t)tw_total * 8 + (size_t)hf_floats * 4 + (size_t)groups * group_bytes;
    }
};
__host__ __device__ inline FiltSmem filt_smem(int p, int tw_total)
{
    FiltSmem f;
    f.tw_total = tw_total;
    f.hf_floats = ((p / 2 + 1) + 3) & ~3;  // 16-byte multiple
    f.group_bytes = 2 * padded_len(p) * 8;
    f.groups = kFiltThreads / fft_threads(p);
    return f;
}

template <typename T> __device__ __forceinline__ T store_cvt(float v);
template <> __device__ __forceinline__ float store_cvt<float>(float v) { return v; }
template <> __device__ __forceinline__ __half store_cvt<__half>(float v) { return __float2half_rn(v); }
template <> __device__ __forceinline__ __nv_bfloat16 store_cvt<__nv_bfloat16>(float v)
{
    return __float2bfloat16_rn(v);
}

// Element offset of output row `row` (= b*H + r) of the raw-sample output.
__device__ __forceinline__ long long out_row_offset(const FiltParams &P, long long row, int &r)
{
    const long long b = row / P.L.H;
    r = (int)(row - b * P.L.H);
    return P.out_layout == TK_LAYOUT_SINOGRAM ? ((long long)r * P.L.N + b) * P.Wp : row * (long long)P.Wp;
}

template <typename T, int LG>
__global__ void __launch_bounds__(kFiltThreads) filter_fft_kernel(const __grid_constant__ FiltParams P)
{
    extern __shared__ __align__(16) float2 fsm[];
    constexpr int p = 1 << LG;
    const FFTPlan &pl = P.plan;
    const FiltSmem lay = filt_smem(p, pl.tw_total);
    constexpr int TPF = fft_threads_c(p);
    constexpr int G = kFiltThreads / TPF;
    const int grp = threadIdx.x / TPF, t = threadIdx.x - grp * TPF;
    float2 *twp = fsm;
    float *hf = reinterpret_cast<float *>(fsm + lay.tw_total);
    float2 *bufA = reinterpret_cast<float2 *>(reinterpret_cast<char *>(hf + lay.hf_floats) + (size_t)grp * lay.group_bytes);
    float2 *bufB = bufA + padded_len(p);
    fill_twiddles(twp, pl);
    for (int k = threadIdx.x; k <= p / 2; k += kFiltThreads) hf[k] = P.Hf[k];
    const float sigma = P.q_scale ? *P.q_scale : 1.f;
    const int W = P.L.W;
    T *out = static_cast<T *>(P.out);
    __syncthreads();

    // Raw samples of a pair group's two rows, fetched one group ahead so that
    // their latency overlaps the transforms of the current one.  Thread t owns
    // the run x0 = t NV .. x0 + NV - 1 of each row (NV TPF = p/2 >= W).
    constexpr int NV = (p / 2 + TPF - 1) / TPF;
    static_assert(NV * TPF >= p / 2, "sample runs must cover the first half of the transform");
    const int x0 = t * NV;
    float raw_a[NV], raw_b[NV];
    auto fetch = [&](long long pgf) {
        const long long pr = pgf * G + grp;
        const bool vl = pr < P.npairs;
        const bool hb = vl && 2 * pr + 1 < P.nrows;
        int rr;
        const long long oa = vl ? in_row_offset(P.L, 2 * pr, rr) : 0;
        const long long ob = hb ? in_row_offset(P.L, 2 * pr + 1, rr) : 0;
        load_run<NV>(P.L, oa, x0, vl, raw_a);
        load_run<NV>(P.L, ob, x0, hb, raw_b);
    };
    if ((long long)blockIdx.x * G < P.npairs) fetch(blockIdx.x);
    for (long long pg = blockIdx.x; pg * G < P.npairs; pg += gridDim.x) {
        const long long pair = pg * G + grp;
        const bool valid = pair < P.npairs;
        const long long ra = 2 * pair, rb = 2 * pair + 1;
        const bool hasb = valid && rb < P.nrows;
        if (valid) {
            int r_a = 0, r_b = 0;
            in_row_offset(P.L, ra, r_a);
            if (hasb) in_row_offset(P.L, rb, r_b);
            const float rta = weight_row_term(P.L, r_a), rtb = weight_row_term(P.L, r_b);
#pragma unroll
            for (int j = 0; j < NV; ++j) {
                const int x = x0 + j;
                if (NV * TPF == p / 2 || x < p / 2)  // short transforms: runs past p/2 are the padding's
                    bufA[pidx(x)] = x < W ? make_float2(pre_from_raw(P.L, r_a, x, raw_a[j], rta),
                                                        hasb ? pre_from_raw(P.L, r_b, x, raw_b[j], rtb) : 0.f)
                                          : make_float2(0.f, 0.f);
            }
            for (int x = p / 2 + t; x < p; x += TPF) bufA[pidx(x)] = make_float2(0.f, 0.f);  // zero padding
        }
        if ((pg + gridDim.x) * G < P.npairs) fetch(pg + gridDim.x);
        group_sync<TPF>(grp);
        float2 *R = fft_forward_c<LG>(bufA, bufB, twp, t, grp);
        float2 *Sb = (R == bufA) ? bufB : bufA;
        // conj(Z) * Hf (Hf real and even)
#pragma unroll 4
        for (int k = t; k < p; k += TPF) {
            const float h = hf[k <= (p >> 1) ? k : p - k];
            const float2 z = R[pidx(k)];
            R[pidx(k)] = make_float2(z.x * h, -z.y * h);
        }
        group_sync<TPF>(grp);
        float2 *Q = fft_forward_c<LG>(R, Sb, twp, t, grp);
        if (valid) {
            int r_a, r_b;
            T *qa = out + out_row_offset(P, ra, r_a);
            const float rta = weight_row_term(P.L, r_a);
            for (int i = t; i < W; i += TPF) {
                const float w = P.weight_out ? cosine_weight_rt(P.L, rta, i) : 1.f;
                qa[i] = store_cvt<T>(Q[pidx(i)].x * sigma * w);
            }
            if (hasb) {
                T *qb = out + out_row_offset(P, rb, r_b);
                const float rtb = weight_row_term(P.L, r_b);
                for (int i = t; i < W; i += TPF) {
                    const float w = P.weight_out ? cosine_weight_rt(P.L, rtb, i) : 1.f;
                    qb[i] = store_cvt<T>(-Q[pidx(i)].y * sigma * w);
                }
            }
        }
        group_sync<TPF>(grp);  // buffers are reused by the next pair group
    }
}

// ---------------------------------------------------------------------------
// Filter straight into a bilinear coefficient image.
//
// A work unit is RC consecutive detector rows of one projection.  The group
// filters the unit's rows two at a time (plus the first row of the next unit,
// which the last coefficient row needs) and keeps the previous filtered row in
// registers (each thread holds it at the columns of its own entries), so
// every coefficient row r is formed from filtered rows r and r+1 without
// another pass over HBM.  Samples outside the detector are 0.

template <int MODE, int LG>
__global__ void __launch_bounds__(kFiltThreads) filter_coef_kernel(const __grid_constant__ FiltParams P)
{
    extern __shared__ __align__(16) float2 fsm[];
    constexpr int p = 1 << LG;
    const FFTPlan &pl = P.plan;
    const FiltSmem lay = filt_smem(p, pl.tw_total);
    constexpr int TPF = fft_threads_c(p);
    constexpr int G = kFiltThreads / TPF;
    const int grp = threadIdx.x / TPF, t = threadIdx.x - grp * TPF;
    float2 *twp = fsm;
    float *hf = reinterpret_cast<float *>(fsm + lay.tw_total);
    float2 *bufA = reinterpret_cast<float2 *>(reinterpret_cast<char *>(hf + lay.hf_floats) + (size_t)grp * lay.group_bytes);
    float2 *bufB = bufA + padded_len(p);
    fill_twiddles(twp, pl);
    for (int k = threadIdx.x; k <= p / 2; k += kFiltThreads) hf[k] = P.Hf[k];
    const float sigma = P.q_scale ? *P.q_scale : 1.f;
    const int W = P.L.W, H = P.L.H, RC = P.rc;
    const int Wc = MODE == TK_F32_COEF ? W : ((W + 1) & ~1);
    __syncthreads();

    for (long long ug = blockIdx.x; ug * G < P.nunits; ug += gridDim.x) {
        const long long unit = ug * G + grp;
        const bool valid = unit < P.nunits;
        const long long b = valid ? unit / P.nchunks : 0;
        const int r0 = valid ? (int)(unit - b * P.nchunks) * RC : 0;
        // the frame of the input and of the output (frame groups: fgrp frames every fstride)
        const long long bf = P.fgrp > 0 ? b / P.fgrp * P.fstride + b % P.fgrp : b;
        const int r1 = min(r0 + RC, H);         // coefficient rows [r0, r1)
        const int rend = min(r0 + RC, H - 1);   // last filtered row (includes the next unit's first)
        const int npair = valid ? (rend - r0 + 2) / 2 : 0;
        // every group runs the same number of pair steps
        const int steps = (min(RC, H - 1) + 2) / 2;
        // Raw samples x0 .. x0 + NV - 1 (x0 = t NV; NV TPF = p/2 >= W) of the
        // next step's two rows, fetched one step ahead so that their latency
        // overlaps the transforms.
        constexpr int NV = (p / 2 + TPF - 1) / TPF;
        static_assert(NV * TPF >= p / 2, "sample runs must cover the first half of the transform");
        const int x0 = t * NV;
        float raw_a[NV], raw_b[NV];
        auto fetch = [&](int kk) {
            const bool lv = valid && kk < npair;
            const int qa = r0 + 2 * kk, qb = qa + 1;
            const bool hb = lv && qb <= rend;
            int rr;
            const long long oa = lv ? in_row_offset(P.L, bf * H + qa, rr) : 0;
            const long long ob = hb ? in_row_offset(P.L, bf * H + qb, rr) : 0;
            load_run<NV>(P.L, oa, x0, lv, raw_a);
            load_run<NV>(P.L, ob, x0, hb, raw_b);
        };
        // The previous filtered row (ra - 1) at the columns c, c+1, c+2 of
        // this thread's column pairs c = 2 (i TPF + t): carried in registers
        // from one step to the next.
        constexpr int NPR = NV / 2 > 0 ? NV / 2 : 1;
        float pv[NPR][3];
#pragma unroll
        for (int i = 0; i < NPR; ++i) pv[i][0] = pv[i][1] = pv[i][2] = 0.f;
        fetch(0);
        for (int k = 0; k < steps; ++k) {
            const bool live = valid && k < npair;
            const int ra = r0 + 2 * k, rb = ra + 1;
            const bool hasb = live && rb <= rend;
            if (live) {
                const float rta = weight_row_term(P.L, ra), rtb = weight_row_term(P.L, rb);
#pragma unroll
                for (int j = 0; j < NV; ++j) {
                    const int x = x0 + j;
                    if (NV * TPF == p / 2 || x < p / 2)  // short transforms: runs past p/2 are the padding's
                        bufA[pidx(x)] = x < W ? make_float2(pre_from_raw(P.L, ra, x, raw_a[j], rta),
                                                            hasb ? pre_from_raw(P.L, rb, x, raw_b[j], rtb) : 0.f)
                                              : make_float2(0.f, 0.f);
                }
                for (int x = p / 2 + t; x < p; x += TPF) bufA[pidx(x)] = make_float2(0.f, 0.f);  // zero padding
            }
            if (k + 1 < steps) fetch(k + 1);
            group_sync<TPF>(grp);
            float2 *R = fft_forward_c<LG>(bufA, bufB, twp, t, grp);
            float2 *Sb = (R == bufA) ? bufB : bufA;
#pragma unroll 4
            for (int kk = t; kk < p; kk += TPF) {
                const float h = hf[kk <= (p >> 1) ? kk : p - kk];
                const float2 z = R[pidx(kk)];
                R[pidx(kk)] = make_float2(z.x * h, -z.y * h);
            }
            group_sync<TPF>(grp);
            const float2 *Q = fft_forward_c<LG>(R, Sb, twp, t, grp);
            if (live) {
                const size_t base = (size_t)bf * H;
                const float zero[3] = {0.f, 0.f, 0.f};
#pragma unroll
                for (int i = 0; i < NPR; ++i) {
                    const int c = 2 * (i * TPF + t);
                    if (c < W) {
                        // rows ra (Re) and rb (-Im) at c, c+1, c+2; columns >= W read as 0
                        float a[3], bb[3];
#pragma unroll
                        for (int k3 = 0; k3 < 3; ++k3) {
                            const float2 q = Q[pidx(c + k3)];
                            const bool in = c + k3 < W;
                            a[k3] = in ? q.x * sigma : 0.f;
                            bb[k3] = in ? -q.y * sigma : 0.f;
                        }
                        if (ra - 1 >= r0)  // prev = row ra-1, next = row ra
                            emit_coef_pair<MODE>(P.out, (base + ra - 1) * Wc, c, W, pv[i], a);
                        if (ra < r1)  // next = row rb, or 0 below the detector's last row
                            emit_coef_pair<MODE>(P.out, (base + ra) * Wc, c, W, a, hasb ? bb : zero);
                        if (hasb && rb < r1 && rb == rend)  // detector's last row, nothing follows
                            emit_coef_pair<MODE>(P.out, (base + rb) * Wc, c, W, bb, zero);
                        if (hasb) {
                            pv[i][0] = bb[0];
                            pv[i][1] = bb[1];
                            pv[i][2] = bb[2];
                        }
                    }
                }
            }
            group_sync<TPF>(grp);  // the buffers are rewritten by the next step
        }
    }
}

// max |preprocessed sample| over the whole input, as float bits in *maxbits.
// Each warp takes whole detector rows (lanes on consecutive columns), so the
// row's offset is formed once per row rather than by a division per sample.
__global__ void __launch_bounds__(256) prescan_kernel(const __grid_constant__ LoadParams L, long long nrows,
                                                      unsigned *maxbits)
{
    float m = 0.f;
    const int lane = threadIdx.x & 31;
    const long long nwarps = ((long long)gridDim.x * blockDim.x) >> 5;
    for (long long row = (blockIdx.x * (long long)blockDim.x + threadIdx.x) >> 5; row < nrows; row += nwarps) {
        int r;
        const long long off = in_row_offset(L, row, r);
        for (int x = lane; x < L.W; x += 32) {
            const float v = fabsf(load_pre(L, off, r, x));
            if (v == v) m = fmaxf(m, v);  // NaN input leaves the bound unchanged
        }
    }
    for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
    __shared__ float wm[8];
    if ((threadIdx.x & 31) == 0) wm[threadIdx.x >> 5] = m;
    __syncthreads();
    if (threadIdx.x == 0) {
        for (int w = 1; w < (int)(blockDim.x >> 5); ++w) m = fmaxf(m, wm[w]);
        atomicMax(maxbits, __float_as_uint(m));
    }
}

// Turns the bound into a power-of-two storage scale: |q| <= max * L1K.  With
// bound = f 2^eb (f in [0.5, 1)), 2^(14 - eb) is the largest power of two s
// with s bound <= 2^14 = kScaleTarget (exact exponent arithmetic, FP32).
__global__ void scale_finalize_kernel(float *scale, float L1K)
{
    const float m = __uint_as_float(*reinterpret_cast<unsigned *>(scale));
    float s = 1.f;
    const float bound = m * L1K * (1.f + 0x1p-20f);  // rounded up past the two FP32 roundings
    if (bound > 0.f && isfinite(bound)) {
        int eb = 0;
        (void)frexpf(bound, &eb);
        const int e = max(-100, min(100, 14 - eb));
        s = ldexpf(1.f, e);
    }
    *scale = s;
}

__global__ void set_scale_kernel(float *scale, float v) { *scale = v; }

// ---------------------------------------------------------------------------
// host: filter spectrum (FP64), cached per (W, tau, window, p)

struct Spectrum {
    int p;
    std::vector<float> Hf;  // p/2 + 1
    double L1K;             // sum_n |K[n]|, K = unnormalised spatial kernel, |n| < W
};

// FilteredBackProjection::RamLak (kernel.cu:792-802), float result.
static float ramlak_ref(int v, float sm)
{
    if (v == 0) return (float)(1. / (4. * sm * sm));
    if ((v % 2) == 0) return 0.f;
    return (float)(-1. / (v * v * M_PI * M_PI * sm * sm));
}

static double window_gain(int window, int k, int p)
{
    const double f = (double)k / (double)p;
    if (window == TK_WINDOW_SHEPP_LOGAN) return k == 0 ? 1.0 : std::sin(M_PI * f) / (M_PI * f);
    if (window == TK_WINDOW_HANN) return 0.5 * (1.0 + std::cos(2.0 * M_PI * f));
    return 1.0;
}

static const Spectrum &spectrum(int W, float tau, int window, int p)
{
    static std::mutex mu;
    static std::map<std::tuple<int, uint32_t, int, int>, Spectrum> cache;
    uint32_t tb;
    std::memcpy(&tb, &tau, 4);
    const auto key = std::make_tuple(W, tb, window, p);
    std::lock_guard<std::mutex> lk(mu);
    auto it = cache.find(key);
    if (it != cache.end()) return it->second;
    Spectrum sp;
    sp.p = p;
    // h[i] = RamLak(i - W/2)/2 for i < W, zero padded (FillFilter, kernel.cu:783-790)
    std::vector<float> h(W);
    for (int i = 0; i < W; ++i) h[i] = ramlak_ref(i - W / 2, tau) / 2;
    std::vector<double> ct(p), st(p);
    for (int m = 0; m < p; ++m) {
        ct[m] = std::cos(2.0 * M_PI * m / p);
        st[m] = std::sin(2.0 * M_PI * m / p);
    }
    std::vector<double> Hd(p / 2 + 1);
    for (int k = 0; k <= p / 2; ++k) {
        double sr = 0, si = 0;
        for (int i = 0; i < W; ++i) {
            const int m = (int)(((long long)k * i) % p);
            sr += h[i] * ct[m];
            si -= h[i] * st[m];
        }
        // AbsKernel: sampling * |X| (kernel.cu:55-64)
        Hd[k] = (double)tau * std::sqrt(sr * sr + si * si) * window_gain(window, k, p);
    }
    sp.Hf.resize(p / 2 + 1);
    for (int k = 0; k <= p / 2; ++k) sp.Hf[k] = (float)Hd[k];
    double L1 = 0;
    for (int n = 0; n < W; ++n) {
        double s = Hd[0] + Hd[p / 2] * ((n & 1) ? -1.0 : 1.0);
        for (int k = 1; k < p / 2; ++k) s += 2.0 * Hd[k] * ct[(int)(((long long)k * n) % p)];
        L1 += (n == 0 ? 1.0 : 2.0) * std::fabs(s);
    }
    sp.L1K = L1;
    return cache.emplace(key, std::move(sp)).first->second;
}

// The kernel instantiated for storage `precision` and pad length 2^lg
// (2 <= lg <= 13; coefficient storage up to lg = 12, i.e. W <= 2048).
template <int LG> static const void *filter_kernel_lg(int precision)
{
    switch (precision) {
    case TK_F32: return reinterpret_cast<const void *>(&filter_fft_kernel<float, LG>);
    case TK_F16: if constexpr (LG <= 12) return reinterpret_cast<const void *>(&filter_coef_kernel<TK_F16, LG>); break;
    case TK_BF16: if constexpr (LG <= 12) return reinterpret_cast<const void *>(&filter_coef_kernel<TK_BF16, LG>); break;
    case TK_F32_COEF:
        if constexpr (LG <= 12) return reinterpret_cast<const void *>(&filter_coef_kernel<TK_F32_COEF, LG>);
        break;
    }
    return nullptr;
}

static const void *filter_kernel_fn(int precision, int lg)
{
    switch (lg) {
    case 2: return filter_kernel_lg<2>(precision);
    case 3: return filter_kernel_lg<3>(precision);
    case 4: return filter_kernel_lg<4>(precision);
    case 5: return filter_kernel_lg<5>(precision);
    case 6: return filter_kernel_lg<6>(precision);
    case 7: return filter_kernel_lg<7>(precision);
    case 8: return filter_kernel_lg<8>(precision);
    case 9: return filter_kernel_lg<9>(precision);
    case 10: return filter_kernel_lg<10>(precision);
    case 11: return filter_kernel_lg<11>(precision);
    case 12: return filter_kernel_lg<12>(precision);
    case 13: return filter_kernel_lg<13>(precision);
    }
    return nullptr;
}

static int launch_filter_typed(const FiltParams &P, int p, cudaStream_t stream, int precision)
{
    const void *fn = filter_kernel_fn(precision, P.lg);
    TK_CHECK(fn, TK_ERR_UNSUPPORTED, "filter: no kernel for pad length %d with this storage", p);
    const int G = kFiltThreads / fft_threads(p);
    const size_t smem = filt_smem(p, P.plan.tw_total).bytes();
    TK_CHECK(smem <= 227 * 1024, TK_ERR_UNSUPPORTED, "filter: pad length %d needs too much shared memory", p);
    TK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0, per_sm = 0;
    TK_CUDA(cudaGetDevice(&dev));
    TK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, fn, kFiltThreads, smem));
    if (per_sm < 1) per_sm = 1;
    const long long work = is_coef(precision) ? P.nunits : P.npairs;
    const long long groups = (work + G - 1) / G;
    const long long grid = std::min<long long>(groups, (long long)sms * per_sm);
    void *args[] = {const_cast<FiltParams *>(&P)};
    TK_CUDA(cudaLaunchKernel(fn, dim3((unsigned)std::max<long long>(grid, 1)), dim3(kFiltThreads), args, smem,
                             stream));
    count_launch();
    return TK_OK;
}

int launch_filter(const tk_geometry &g, const void *d_in, int input_type, int layout, const tk_flatfield *ff,
                  int window, void *d_q, int precision, float *d_q_scale, cudaStream_t stream, int fgrp, int fstride,
                  int form)
{
    if (int rc = validate_geometry(&g)) return rc;
    TK_CHECK(fgrp <= 0 || (is_coef(precision) && layout == TK_LAYOUT_PROJECTION && fstride >= fgrp), TK_ERR_INVALID,
             "filter: frame groups need a coefficient image from detector frames");
    TK_CHECK(d_in && d_q, TK_ERR_INVALID, "filter: null device pointer");
    TK_CHECK(input_type == TK_INPUT_F32 || input_type == TK_INPUT_U16, TK_ERR_INVALID, "filter: bad input type");
    TK_CHECK(layout == TK_LAYOUT_SINOGRAM || layout == TK_LAYOUT_PROJECTION, TK_ERR_INVALID, "filter: bad layout");
    TK_CHECK(window >= TK_WINDOW_RAMLAK && window <= TK_WINDOW_HANN, TK_ERR_INVALID, "filter: bad window");
    TK_CHECK(valid_precision(precision), TK_ERR_INVALID, "filter: bad precision");
    const bool sixteen = precision == TK_F16 || precision == TK_BF16;
    TK_CHECK(!sixteen || d_q_scale, TK_ERR_INVALID, "filter: 16-bit storage needs d_q_scale");
    TK_CHECK(fgrp <= 0 || !sixteen || (input_type == TK_INPUT_U16 && ff && !ff->dark && !ff->flat), TK_ERR_INVALID,
             "filter: frame groups need a storage scale known without a scan of the data");
    TK_CHECK(input_type == TK_INPUT_F32 || ff, TK_ERR_INVALID, "filter: raw input needs flat-field parameters");
    const int p = reference_pad_length(g.W);
    TK_CHECK(p <= 2 * (kMaxHf - 1), TK_ERR_UNSUPPORTED, "filter: W = %d exceeds the supported 4096", g.W);
    TK_CHECK(!is_coef(precision) || p <= 4096, TK_ERR_UNSUPPORTED,
             "filter: coefficient storage supports W <= 2048 (W = %d)", g.W);

    static thread_local FiltParams P;  // ~16 KB: keep off the stack
    std::memset(&P, 0, sizeof(P));
    LoadParams &L = P.L;
    L.in = d_in;
    L.W = g.W;
    L.N = g.N;
    L.H = g.H;
    L.layout = layout;
    L.input_type = input_type;
    L.in_pitch = g.W;
    L.weight_in = 1;
    L.cX = g.cX;
    L.cZ = g.cZ;
    L.D = g.D;
    L.A = 1.f;
    if (input_type == TK_INPUT_U16) {
        TK_CHECK(ff->floor_counts > 0.f, TK_ERR_INVALID, "filter: floor_counts must be > 0");
        TK_CHECK(ff->flat || ff->flat_value > 0.f, TK_ERR_INVALID, "filter: flat field missing");
        L.dark = ff->dark;
        L.flat = ff->flat;
        L.dark_v = ff->dark_value;
        L.flat_v = ff->flat_value;
        L.A = ff->A;
        L.B = ff->B;
        L.invert = ff->invert ? 1 : 0;
        L.floor_counts = ff->floor_counts;
    }
    finish_load_params(L);
    const Spectrum &sp = spectrum(g.W, g.tau, window, p);
    P.out = d_q;
    P.out_layout = TK_LAYOUT_PROJECTION;
    P.weight_out = 0;
    P.nrows = (long long)g.N * g.H;
    P.npairs = (P.nrows + 1) / 2;
    P.Wp = row_pitch(g.W);
    P.p = p;
    int lg = 0;
    while ((1 << lg) < p) ++lg;
    P.lg = lg;
    P.plan = fft_plan(lg);
    P.precision = precision;
    P.rc = 64;
    P.nchunks = (g.H + P.rc - 1) / P.rc;
    P.nunits = (long long)g.N * P.nchunks;
    P.fgrp = fgrp > 0 ? fgrp : 0;
    P.fstride = fgrp > 0 ? fstride : 0;
    std::memcpy(P.Hf, sp.Hf.data(), sizeof(float) * sp.Hf.size());

    if (!sixteen) {
        P.q_scale = nullptr;
        if (d_q_scale) {
            set_scale_kernel<<<1, 1, 0, stream>>>(d_q_scale, 1.f);
            count_launch();
        }
    } else if (input_type == TK_INPUT_U16 && !ff->dark && !ff->flat) {
        // Scalar flat/dark: |A log(num/den) + B| is bounded without looking at the
        // data, since num in [floor, 65535] and den = max(flat - dark, floor).
        const double fl = ff->floor_counts, den = std::fmax((double)ff->flat_value - ff->dark_value, fl);
        const double lg = std::fmax(std::fabs(std::log(fl / den)), std::fabs(std::log(65535.0 / fl)));
        const double bound = (std::fabs((double)ff->A) * lg + std::fabs((double)ff->B)) * sp.L1K;
        int e = bound > 0 ? (int)std::floor(std::log2((double)kScaleTarget / bound)) : 0;
        e = std::max(-100, std::min(100, e));
        set_scale_kernel<<<1, 1, 0, stream>>>(d_q_scale, (float)std::ldexp(1.0, e));
        count_launch();
        P.q_scale = d_q_scale;
    } else {
        TK_CUDA(cudaMemsetAsync(d_q_scale, 0, sizeof(float), stream));
        int dev = 0, sms = 0;
        TK_CUDA(cudaGetDevice(&dev));
        TK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
        prescan_kernel<<<sms * 4, 256, 0, stream>>>(L, P.nrows, reinterpret_cast<unsigned *>(d_q_scale));
        scale_finalize_kernel<<<1, 1, 0, stream>>>(d_q_scale, (float)sp.L1K);
        count_launch(2);  // prescan + finalize
        P.q_scale = d_q_scale;
    }
    TK_CUDA(cudaGetLastError());
    const int use = form <= TK_FILTER_AUTO ? filter_form_for(g.W, precision)
                    : (form == TK_FILTER_TOEPLITZ && toeplitz_supported(g.W, precision, TK_LAYOUT_PROJECTION))
                        ? TK_FILTER_TOEPLITZ
                        : TK_FILTER_FFT;
    if (use == TK_FILTER_TOEPLITZ)
        return launch_filter_toeplitz(L, P.Hf, p, d_q, precision, P.q_scale, P.nrows, storage_pitch(g.W, precision),
                                      P.fgrp, P.fstride, stream);
    return launch_filter_typed(P, p, stream, precision);
}

// Filter form selection (tk_filter_select_form).  TK_FILTER_AUTO takes the
// tensor-core Toeplitz product for 16-bit storage up to kToeplitzAutoMaxW,
// where it measured faster than the FFT (360 uint16 frames into FP16
// coefficients: 2.2x at W = 128, 1.5x at 192, 1.4x at 256 and 384, 1.1x at
// 512), and the FFT otherwise.  FP32 storage keeps the FFT: the split-BF16
// product carries about 2e-5 relative error on the filtered values, below
// 16-bit storage rounding (2^-12 or coarser) but above the FP32 forms' 1e-5
// reconstruction bound.
static int g_filter_form = TK_FILTER_AUTO;
constexpr int kToeplitzAutoMaxW = 512;

int filter_form_for(int W, int precision)
{
    const bool ok = toeplitz_supported(W, precision, TK_LAYOUT_PROJECTION);
    if (g_filter_form == TK_FILTER_TOEPLITZ) return ok ? TK_FILTER_TOEPLITZ : TK_FILTER_FFT;
    if (g_filter_form == TK_FILTER_FFT) return TK_FILTER_FFT;
    const bool sixteen = precision == TK_F16 || precision == TK_BF16;
    return ok && sixteen && W <= kToeplitzAutoMaxW ? TK_FILTER_TOEPLITZ : TK_FILTER_FFT;
}

// Transpose of the filter stage for the adjoint: the ramp filter is a
// symmetric Toeplitz operator (its spectrum is real and even) and the cosine
// weight is diagonal, so (F W)^T = W F.  Reads a [N][H][Wp] FP32 gradient,
// filters each row with the same spectrum and unnormalised scale, multiplies
// by the cosine weight and writes FP32 in `layout` with row pitch W.
int launch_filter_transpose(const tk_geometry &g, const float *d_qbar, int window, float *d_pbar, int layout,
                            cudaStream_t stream)
{
    if (int rc = validate_geometry(&g)) return rc;
    TK_CHECK(d_qbar && d_pbar, TK_ERR_INVALID, "filter transpose: null device pointer");
    TK_CHECK(layout == TK_LAYOUT_SINOGRAM || layout == TK_LAYOUT_PROJECTION, TK_ERR_INVALID, "bad layout");
    TK_CHECK(window >= TK_WINDOW_RAMLAK && window <= TK_WINDOW_HANN, TK_ERR_INVALID, "bad window");
    const int p = reference_pad_length(g.W);
    TK_CHECK(p <= 2 * (kMaxHf - 1), TK_ERR_UNSUPPORTED, "filter: W = %d exceeds the supported 4096", g.W);
    static thread_local FiltParams P;
    std::memset(&P, 0, sizeof(P));
    LoadParams &L = P.L;
    L.in = d_qbar;
    L.W = g.W;
    L.N = g.N;
    L.H = g.H;
    L.layout = TK_LAYOUT_PROJECTION;
    L.input_type = TK_INPUT_F32;
    L.in_pitch = row_pitch(g.W);
    L.weight_in = 0;
    L.cX = g.cX;
    L.cZ = g.cZ;
    L.D = g.D;
    L.A = 1.f;
    finish_load_params(L);
    const Spectrum &sp = spectrum(g.W, g.tau, window, p);
    P.out = d_pbar;
    P.out_layout = layout;
    P.weight_out = 1;
    P.q_scale = nullptr;
    P.nrows = (long long)g.N * g.H;
    P.npairs = (P.nrows + 1) / 2;
    P.Wp = g.W;  // dense output rows
    P.p = p;
    int lg = 0;
    while ((1 << lg) < p) ++lg;
    P.lg = lg;
    P.plan = fft_plan(lg);
    P.precision = TK_F32;
    std::memcpy(P.Hf, sp.Hf.data(), sizeof(float) * sp.Hf.size());
    return launch_filter_typed(P, p, stream, TK_F32);
}

}  // namespace tk

extern "C" int tk_filter_select_form(int form)
{
    if (form < TK_FILTER_AUTO || form > TK_FILTER_TOEPLITZ) {
        tk::set_error("no filter form %d", form);
        return TK_ERR_INVALID;
    }
    tk::g_filter_form = form;
    return TK_OK;
}

extern "C" int tk_filter_form_for(int W, int precision) { return tk::filter_form_for(W, precision); }
