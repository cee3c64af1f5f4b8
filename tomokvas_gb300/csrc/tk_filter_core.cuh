// tk_filter_core.cuh -- device pieces shared by the ramp-filter kernels
// (the shared-memory FFT in tk_filter.cu, the tensor-core Toeplitz product in
// tk_toeplitz.cu): the raw-input description, the fused preprocessing of a
// sample (flat field + log, cosine weight) and the coefficient-entry writer.
#pragma once

#include "tk_common.cuh"

namespace tk {

struct LoadParams {
    const void *in;
    const float *dark, *flat;
    float dark_v, flat_v, A, B, floor_counts;
    int invert;
    int W, N, H, layout, input_type;
    int in_pitch;   // elements between consecutive input rows of one layout line (W, or Wp)
    int weight_in;  // apply the cosine weight while loading (forward); 0 for the transpose
    float cX, cZ, D;
    float D2;       // D * D
    float inv_den;  // 1 / max(flat - dark, floor) for scalar flat/dark
    int vec;        // rows start 16-byte aligned and span whole 16-byte chunks: chunked loads
};

// Element offset of the first sample of output row `row` (= b*H + r) in the input.
__device__ __forceinline__ long long in_row_offset(const LoadParams &L, long long row, int &r)
{
    const long long b = row / L.H;
    r = (int)(row - b * L.H);
    return L.layout == TK_LAYOUT_SINOGRAM ? ((long long)r * L.N + b) * L.in_pitch : row * (long long)L.in_pitch;
}

// row[x] *= distance / sqrt(ce*ce + distance*distance + cs*cs)  (kernel.cu:195-199),
// evaluated as D rsqrt(ce^2 + (cs^2 + D^2)) with the row term cs^2 + D^2
// formed once per row (within 2 ulp of the IEEE divide and square root).
__device__ __forceinline__ float weight_row_term(const LoadParams &L, int r)
{
    const float cs = (float)r - L.cZ;
    return fmaf(cs, cs, L.D2);
}
__device__ __forceinline__ float cosine_weight_rt(const LoadParams &L, float rt, int x)
{
    const float ce = (float)x - L.cX;
    return L.D * rsqrtf(fmaf(ce, ce, rt));
}

// Raw sample x of the row at element offset off (counts as float for u16).
__device__ __forceinline__ float load_raw(const LoadParams &L, long long off, int x)
{
    return L.input_type == TK_INPUT_U16 ? (float)static_cast<const uint16_t *>(L.in)[off + x]
                                        : static_cast<const float *>(L.in)[off + x];
}

// Preprocessing of a raw sample: flat-field + log if raw counts
// (rsq_load.cpp:299-325: A log(num / den) + B, num = max(I - dark, floor),
// den = max(flat - dark, floor); here in FP32 with __logf, absolute error
// below 4e-7 for transmissions near 1), then the cosine weight (kernel.cu:
// 195-199).  rt is the row's weight_row_term.
__device__ __forceinline__ float pre_from_raw(const LoadParams &L, int r, int x, float raw, float rt)
{
    float val = raw;
    if (L.input_type == TK_INPUT_U16) {
        float t;
        if (L.dark || L.flat) {
            const size_t px = (size_t)r * L.W + x;
            const float dk = L.dark ? L.dark[px] : L.dark_v;
            const float fl = L.flat ? L.flat[px] : L.flat_v;
            t = __fdividef(fmaxf(raw - dk, L.floor_counts), fmaxf(fl - dk, L.floor_counts));
        } else {
            t = fmaxf(raw - L.dark_v, L.floor_counts) * L.inv_den;
        }
        val = fmaf(L.A, __logf(t), L.B);
        if (L.invert) val = -val;
    }
    if (!L.weight_in) return val;
    return val * cosine_weight_rt(L, rt, x);
}

// Preprocessed (log if raw, cosine weighted) sample x of a row.
__device__ __forceinline__ float load_pre(const LoadParams &L, long long off, int r, int x)
{
    return pre_from_raw(L, r, x, load_raw(L, off, x), weight_row_term(L, r));
}

// Coefficient entries of columns c and c+1 of one row (c even, c < W) from
// the row's filtered values a and the next row's b at c, c+1, c+2 (0 at
// columns >= W).  The 16-bit formats store both entries with one 16-byte
// store: their rows hold an even number of entries (Wc), so entry c+1 exists
// and c starts a 16-byte unit; the FP32 format writes entry c+1 only below W.
template <int MODE>
__device__ __forceinline__ void emit_coef_pair(void *img, size_t row_base, int c, int W, const float *a,
                                               const float *b)
{
    const float dU0 = a[1] - a[0], dU1 = a[2] - a[1];
    const float Q0 = a[0], dV0 = b[0] - a[0], dUV0 = (b[1] - b[0]) - dU0;
    const float Q1 = a[1], dV1 = b[1] - a[1], dUV1 = (b[2] - b[1]) - dU1;
    if constexpr (MODE == TK_F32_COEF) {
        float4 *e = static_cast<float4 *>(img) + row_base + c;
        e[0] = make_float4(Q0, dU0, dV0, dUV0);
        if (c + 1 < W) e[1] = make_float4(Q1, dU1, dV1, dUV1);
    } else {
        uint4 e;
        if constexpr (MODE == TK_F16) {
            const __half2 l0 = __floats2half2_rn(Q0, dV0), h0 = __floats2half2_rn(dU0, dUV0);
            const __half2 l1 = __floats2half2_rn(Q1, dV1), h1 = __floats2half2_rn(dU1, dUV1);
            e = make_uint4(*reinterpret_cast<const uint32_t *>(&l0), *reinterpret_cast<const uint32_t *>(&h0),
                           *reinterpret_cast<const uint32_t *>(&l1), *reinterpret_cast<const uint32_t *>(&h1));
        } else {
            const __nv_bfloat162 l0 = __floats2bfloat162_rn(Q0, dV0), h0 = __floats2bfloat162_rn(dU0, dUV0);
            const __nv_bfloat162 l1 = __floats2bfloat162_rn(Q1, dV1), h1 = __floats2bfloat162_rn(dU1, dUV1);
            e = make_uint4(*reinterpret_cast<const uint32_t *>(&l0), *reinterpret_cast<const uint32_t *>(&h0),
                           *reinterpret_cast<const uint32_t *>(&l1), *reinterpret_cast<const uint32_t *>(&h1));
        }
        *reinterpret_cast<uint4 *>(static_cast<uint2 *>(img) + row_base + c) = e;
    }
}

// Derived load parameters: D^2, the scalar flat-field reciprocal, and whether
// rows can be read in 16-byte chunks (aligned base, row pitch a multiple of
// 16 bytes, so every chunk that starts below W lies inside its row).
inline void finish_load_params(LoadParams &L)
{
    L.D2 = L.D * L.D;
    L.inv_den = 1.f;
    if (L.input_type == TK_INPUT_U16 && !L.dark && !L.flat)
        L.inv_den = 1.f / std::fmax(L.flat_v - L.dark_v, L.floor_counts);
    const int es = L.input_type == TK_INPUT_U16 ? 2 : 4;
    L.vec = (reinterpret_cast<uintptr_t>(L.in) % 16 == 0) && ((long long)L.in_pitch * es) % 16 == 0;
}

}  // namespace tk
