// tk_bp.cu -- voxel-driven FDK backprojection for GB300 (sm_103a).
//
// Computes, for every voxel inside the field-of-view cylinder, the FDK sum of
// FBPConeKernel + fQ3D (Lukas-kV/TomoKvas FBPG/kernel.cu:68-177):
//
//   vol = (dfi/p) * sum_b U^2 * Q_b(T*U + cX, aZ*U + cZ),
//   S = aX cos b + aY sin b,  T = aY cos b - aX sin b,  U = D / (D - S),
//
// where Q_b is the zero-outside bilinear interpolation of projection b.
//
// GB300 design:
//  * one CTA owns a TX x TY x TZ voxel tile; each thread owns one (x, y)
//    column and walks TZ voxels along z -- u, U and U^2 are fixed along the
//    column, so the per-update work is one v, one floor/frac, the gathers and
//    three FMAs;
//  * the per-projection cos/sin table lives in the kernel's parameter space
//    (constant bank), one uniform load per column-angle;
//  * for every projection the tile's footprint (bounding box of the 8 tile
//    corners' projections) is staged into shared memory by a plain per-CTA
//    TMA load (cp.async.bulk.tensor.3d, zero fill outside the detector) into
//    a ring of STAGES buffers guarded by mbarriers;
//  * FP32 storage interpolates straight from the staged tile (4 LDS.32 per
//    update); FP16/BF16 storage first expands the staged tile into bilinear
//    coefficient pairs {(Q, dV), (dU, dUV)} so that one LDS.64 + one packed
//    HFMA2 give the two row interpolants, halving shared-memory traffic;
//  * accumulation is FP32 in registers; each voxel is written once.
#include "tk_common.cuh"
#include "tk_internal.h"

#include <cmath>
#include <cstdio>
#include <cstring>
#include <vector>
#include <cudaTypedefs.h>

namespace tk {

constexpr int kMaxParamProj = 3200;  // cos/sin pairs carried in the kernel parameters

struct BPParams {
    float *vol;
    unsigned *err;
    long long slice_stride;  // X * Y
    int X, Y, nz, N;
    int BW, BH;              // staged box (elements)
    int stage_elems;         // elements per raw stage (>= BW*BH, padded)
    int coef_stride;         // coefficient entries per coefficient buffer
    int tilesX;
    int accumulate;
    float cX, cZ, D;
    float dX, dY, zoff, scale;
    unsigned dirx, diry, dirz;  // 0 or 0x80000000 (sign flip, kernel.cu:86-88)
    float Wm1, Hm1;             // W-1, H-1
    double halfW;               // W / 2. (kernel.cu:100)
    float fscale;               // dfi * (1/p)  (kernel.cu:113)
    const float *q_scale;       // device storage scale of the filtered projections, or null (= 1)
    float2 trig[kMaxParamProj]; // (cos, sin) per projection (kernel.cu:430-441)
};

__device__ __forceinline__ float flip(float v, unsigned mask)
{
    return __uint_as_float(__float_as_uint(v) ^ mask);
}

// Storage traits -------------------------------------------------------------
struct StoreF32 {
    using T = float;
    static constexpr int kAlign = 4;  // TMA x coordinate granularity (16 B)
    static constexpr bool kCoef = false;
};
struct StoreF16 {
    using T = __half;
    static constexpr int kAlign = 8;
    static constexpr bool kCoef = true;
};
struct StoreBF16 {
    using T = __nv_bfloat16;
    static constexpr int kAlign = 8;
    static constexpr bool kCoef = true;
};

// Bounding box origin of the footprint of tile (x0,y0,z0) in projection b.
template <int TX, int TY, int TZ, int ALIGN>
__device__ __forceinline__ int2 footprint_origin(const BPParams &P, int b, int x0, int y0, int z0)
{
    const float2 cs = P.trig[b];
    const int xs[2] = {x0, min(x0 + TX - 1, P.X - 1)};
    const int ys[2] = {y0, min(y0 + TY - 1, P.Y - 1)};
    const int zs[2] = {z0, min(z0 + TZ - 1, P.nz - 1)};
    float aZc[2];
#pragma unroll
    for (int k = 0; k < 2; ++k) aZc[k] = flip(P.scale * ((float)zs[k] + P.zoff), P.dirz);
    float umin = 3.0e38f, vmin = 3.0e38f;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float aX = flip(P.scale * ((float)xs[i] + P.dX), P.dirx);
            const float aY = flip(P.scale * ((float)ys[j] + P.dY), P.diry);
            const float S = aX * cs.x + aY * cs.y;
            const float T = aY * cs.x - aX * cs.y;
            const float U = P.D / (P.D - S);
            umin = fminf(umin, T * U + P.cX);
#pragma unroll
            for (int k = 0; k < 2; ++k) vmin = fminf(vmin, aZc[k] * U + P.cZ);
        }
    }
    int bx = (int)floorf(umin) - 1;
    bx &= ~(ALIGN - 1);  // round down to the TMA granularity (two's complement)
    const int by = (int)floorf(vmin) - 1;
    return make_int2(bx, by);
}

constexpr uint64_t kWaitLimitNs = 2000000000ull;  // 2 s: a TMA stage never takes this long

// ---------------------------------------------------------------------------
// Expansion of a staged 16-bit tile into bilinear coefficient pairs.
// Entry (r, c): lo = (Q, dV), hi = (dU, dUV) with
//   Q = q[r][c], dU = q[r][c+1]-Q, dV = q[r+1][c]-Q, dUV = q[r+1][c+1]-q[r+1][c]-dU,
// so that [top, bot-top] = hi * fu + lo.
template <typename V2>
__device__ __forceinline__ V2 v2_shift(V2 a, V2 b)  // (a.y, b.x)
{
    uint32_t ua = *reinterpret_cast<uint32_t *>(&a), ub = *reinterpret_cast<uint32_t *>(&b);
    uint32_t r = __byte_perm(ua, ub, 0x5432);
    return *reinterpret_cast<V2 *>(&r);
}
template <typename V2>
__device__ __forceinline__ uint32_t v2_bits(V2 a) { return *reinterpret_cast<uint32_t *>(&a); }

template <typename T, typename V2, int NT>
__device__ __forceinline__ void expand_tile(const T *__restrict__ raw, uint2 *__restrict__ coef, int BW, int BH,
                                            int tid)
{
    // Work item = (column pair, band of kBand coefficient rows); walking down
    // the band reuses the previous raw row.
    constexpr int kBand = 4;
    const int npairs = BW >> 1;
    const int nrows = BH - 1;
    const int nbands = (nrows + kBand - 1) / kBand;
    const V2 *raw2 = reinterpret_cast<const V2 *>(raw);
    const int w2 = BW >> 1;  // pairs per raw row
    for (int item = tid; item < npairs * nbands; item += NT) {
        const int pr = item % npairs, band = item / npairs;
        const int r0 = band * kBand;
        const int r1 = min(r0 + kBand, nrows);
        // row r0: columns (2pr, 2pr+1) and (2pr+2, 2pr+3); the second pair of
        // the last column pair lies one element past the row and is never used.
        V2 a0 = raw2[r0 * w2 + pr];
        V2 a1 = raw2[r0 * w2 + pr + 1];
        V2 dU0 = __hsub2(v2_shift(a0, a1), a0);
        for (int r = r0; r < r1; ++r) {
            const V2 b0 = raw2[(r + 1) * w2 + pr];
            const V2 b1 = raw2[(r + 1) * w2 + pr + 1];
            const V2 dU1 = __hsub2(v2_shift(b0, b1), b0);
            const V2 dV = __hsub2(b0, a0);
            const V2 dUV = __hsub2(dU1, dU0);
            // entry (r, 2pr): lo=(a0.x, dV.x) hi=(dU0.x, dUV.x); entry (r, 2pr+1): .y halves
            uint4 out;
            out.x = __byte_perm(v2_bits(a0), v2_bits(dV), 0x5410);
            out.y = __byte_perm(v2_bits(dU0), v2_bits(dUV), 0x5410);
            out.z = __byte_perm(v2_bits(a0), v2_bits(dV), 0x7632);
            out.w = __byte_perm(v2_bits(dU0), v2_bits(dUV), 0x7632);
            *reinterpret_cast<uint4 *>(coef + r * BW + 2 * pr) = out;
            a0 = b0;
            dU0 = dU1;
        }
    }
}

template <typename V2>
__device__ __forceinline__ float2 coef_eval(uint2 c, V2 fu2);

template <>
__device__ __forceinline__ float2 coef_eval<__half2>(uint2 c, __half2 fu2)
{
    const __half2 lo = *reinterpret_cast<__half2 *>(&c.x);
    const __half2 hi = *reinterpret_cast<__half2 *>(&c.y);
    return __half22float2(__hfma2(hi, fu2, lo));
}

template <>
__device__ __forceinline__ float2 coef_eval<__nv_bfloat162>(uint2 c, __nv_bfloat162 fu2)
{
    const __nv_bfloat162 lo = *reinterpret_cast<__nv_bfloat162 *>(&c.x);
    const __nv_bfloat162 hi = *reinterpret_cast<__nv_bfloat162 *>(&c.y);
    return __bfloat1622float2(__hfma2(hi, fu2, lo));
}

template <typename V2> __device__ __forceinline__ V2 splat(float f);
template <> __device__ __forceinline__ __half2 splat<__half2>(float f) { return __float2half2_rn(f); }
template <> __device__ __forceinline__ __nv_bfloat162 splat<__nv_bfloat162>(float f)
{
    return __float2bfloat162_rn(f);
}

template <typename S> struct Vec2Of;
template <> struct Vec2Of<StoreF16> { using type = __half2; };
template <> struct Vec2Of<StoreBF16> { using type = __nv_bfloat162; };
template <> struct Vec2Of<StoreF32> { using type = float2; };

// ---------------------------------------------------------------------------
template <typename S, int TX, int TY, int TZ, int STAGES, int MINB>
__global__ void __launch_bounds__(TX *TY, MINB)
    bp_tma_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ BPParams P)
{
    using T = typename S::T;
    using V2 = typename Vec2Of<S>::type;
    constexpr int NT = TX * TY;
    extern __shared__ __align__(128) unsigned char smem[];

    T *stages = reinterpret_cast<T *>(smem);
    // coefficient buffers (16-bit storage only), 16-byte aligned
    uint2 *coef = reinterpret_cast<uint2 *>(smem + (size_t)STAGES * P.stage_elems * sizeof(T));
    int2 *boxo = reinterpret_cast<int2 *>(reinterpret_cast<unsigned char *>(coef) +
                                          (S::kCoef ? 2 * (size_t)P.coef_stride * sizeof(uint2) : 0));
    uint64_t *full = reinterpret_cast<uint64_t *>(boxo + P.N);
    volatile int &s_abort = *reinterpret_cast<int *>(full + STAGES);

    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int x0 = (blockIdx.x % P.tilesX) * TX, y0 = (blockIdx.x / P.tilesX) * TY;
    const int z0 = blockIdx.y * TZ;
    const int x = x0 + tx, y = y0 + ty;

    const float aX = flip(P.scale * ((float)x + P.dX), P.dirx);
    const float aY = flip(P.scale * ((float)y + P.dY), P.diry);
    const bool inside = (x < P.X) && (y < P.Y);
    const bool active = inside && (sqrtf(aX * aX + aY * aY) < P.halfW);

    if (!__syncthreads_or(active)) {  // tile entirely outside the FOV cylinder
        if (inside) {
            for (int z = 0; z < TZ; ++z) {
                if (z0 + z >= P.nz) break;
                float *dst = P.vol + (size_t)(z0 + z) * P.slice_stride + (size_t)y * P.X + x;
                *dst = P.accumulate ? 0.f + *dst : 0.f;
            }
        }
        return;
    }

    for (int b = tid; b < P.N; b += NT) boxo[b] = footprint_origin<TX, TY, TZ, S::kAlign>(P, b, x0, y0, z0);
    if (tid == 0) {
        s_abort = 0;
        for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
        prefetch_tensormap(&tmap);
    }
    __syncthreads();
    const uint32_t stage_bytes = (uint32_t)(P.BW * P.BH * sizeof(T));
    if (tid == 0) {
        for (int s = 0; s < STAGES && s < P.N; ++s) {
            mbar_arrive_expect_tx(&full[s], stage_bytes);
            tma_load_3d(stages + (size_t)s * P.stage_elems, &tmap, boxo[s].x, boxo[s].y, s, &full[s]);
        }
    }

    // Slices past the end of the slab repeat the last one: their footprint is
    // then inside the staged box and their (unstored) sums are harmless.
    float aZ[TZ];
#pragma unroll
    for (int z = 0; z < TZ; ++z) aZ[z] = flip(P.scale * ((float)min(z0 + z, P.nz - 1) + P.zoff), P.dirz);
    float acc[TZ];
#pragma unroll
    for (int z = 0; z < TZ; ++z) acc[z] = 0.f;

    const float cZ = P.cZ, Hm1 = P.Hm1;
    const uint32_t BW = (uint32_t)P.BW;
    int b = 0;
    for (; b < P.N; ++b) {
        const int s = b % STAGES;
        const uint32_t parity = (uint32_t)(b / STAGES) & 1u;
        const bool got = mbar_wait_bounded(&full[s], parity, kWaitLimitNs);
        if (!got) {
            atomicOr(P.err, ERR_WAIT_TIMEOUT);
            s_abort = 1;
        }
        const int bx0 = boxo[b].x, by0 = boxo[b].y;
        const uint2 *cb_tile = coef + (size_t)(b & 1) * P.coef_stride;
        if constexpr (S::kCoef) {
            if (got) expand_tile<T, V2, NT>(stages + (size_t)s * P.stage_elems, const_cast<uint2 *>(cb_tile),
                                            P.BW, P.BH, tid);
            __syncthreads();
            if (s_abort) break;
            if (tid == 0 && b + STAGES < P.N) {  // raw stage s is free again
                mbar_arrive_expect_tx(&full[s], stage_bytes);
                tma_load_3d(stages + (size_t)s * P.stage_elems, &tmap, boxo[b + STAGES].x, boxo[b + STAGES].y,
                            b + STAGES, &full[s]);
            }
        }
        if (active && got) {
            const float2 cs = P.trig[b];
            const float dcos = cs.x, dsin = cs.y;
            const float Sd = aX * dcos + aY * dsin;
            const float Td = aY * dcos - aX * dsin;
            const float U = P.D / (P.D - Sd);
            const float u = Td * U + P.cX;
            if (u >= 0.f && u <= P.Wm1) {  // column inside the detector (kernel.cu:127-128)
                const float U2 = U * U;
                const float fla = __fadd_rd(u, kMagic);
                const int a = __float_as_int(fla) - kMagicBits;
                const float fu = u - (fla - kMagic);
                const int col = a - bx0;
                const float vA = aZ[0] * U + cZ, vB = aZ[TZ - 1] * U + cZ;
                const float vlo = fminf(vA, vB), vhi = fmaxf(vA, vB);
                const int rlo = (int)floorf(vlo) - by0, rhi = (int)floorf(vhi) + 1 - by0;
                if (col >= 0 && col + 1 < P.BW && rlo >= 0 && rhi < P.BH) {
                    const uint32_t cbase = (uint32_t)col - (uint32_t)(kMagicBits + by0) * BW;
                    const bool all_in = (vlo >= 0.f) && (vhi <= Hm1);
                    if constexpr (!S::kCoef) {
                        const float *st = reinterpret_cast<const float *>(stages) + (size_t)s * P.stage_elems;
                        if (all_in) {
#pragma unroll
                            for (int z = 0; z < TZ; ++z) {
                                const float v = aZ[z] * U + cZ;
                                const float fl = __fadd_rd(v, kMagic);
                                const float fv = v - (fl - kMagic);
                                const uint32_t o = (uint32_t)__float_as_int(fl) * BW + cbase;
                                const float q00 = st[o], q01 = st[o + 1];
                                const float q10 = st[o + BW], q11 = st[o + BW + 1];
                                const float top = fmaf(fu, q01 - q00, q00);
                                const float bot = fmaf(fu, q11 - q10, q10);
                                acc[z] = fmaf(U2, fmaf(fv, bot - top, top), acc[z]);
                            }
                        } else {
#pragma unroll
                            for (int z = 0; z < TZ; ++z) {
                                const float v = aZ[z] * U + cZ;
                                const float fl = __fadd_rd(v, kMagic);
                                const float fv = v - (fl - kMagic);
                                const uint32_t o = (uint32_t)__float_as_int(fl) * BW + cbase;
                                const float q00 = st[o], q01 = st[o + 1];
                                const float q10 = st[o + BW], q11 = st[o + BW + 1];
                                const float top = fmaf(fu, q01 - q00, q00);
                                const float bot = fmaf(fu, q11 - q10, q10);
                                const float w = (v >= 0.f && v <= Hm1) ? U2 : 0.f;  // kernel.cu:130-131
                                acc[z] = fmaf(w, fmaf(fv, bot - top, top), acc[z]);
                            }
                        }
                    } else {
                        const V2 fu2 = splat<V2>(fu);
                        if (all_in) {
#pragma unroll
                            for (int z = 0; z < TZ; ++z) {
                                const float v = aZ[z] * U + cZ;
                                const float fl = __fadd_rd(v, kMagic);
                                const float fv = v - (fl - kMagic);
                                const uint32_t o = (uint32_t)__float_as_int(fl) * BW + cbase;
                                const float2 tb = coef_eval<V2>(cb_tile[o], fu2);
                                acc[z] = fmaf(U2, fmaf(fv, tb.y, tb.x), acc[z]);
                            }
                        } else {
#pragma unroll
                            for (int z = 0; z < TZ; ++z) {
                                const float v = aZ[z] * U + cZ;
                                const float fl = __fadd_rd(v, kMagic);
                                const float fv = v - (fl - kMagic);
                                const uint32_t o = (uint32_t)__float_as_int(fl) * BW + cbase;
                                const float2 tb = coef_eval<V2>(cb_tile[o], fu2);
                                const float w = (v >= 0.f && v <= Hm1) ? U2 : 0.f;
                                acc[z] = fmaf(w, fmaf(fv, tb.y, tb.x), acc[z]);
                            }
                        }
                    }
                } else {
                    atomicOr(P.err, ERR_BOX_OVERFLOW);
                }
            }
        }
        if constexpr (!S::kCoef) {
            __syncthreads();  // every thread is done with stage s
            if (s_abort) break;
            if (tid == 0 && b + STAGES < P.N) {
                mbar_arrive_expect_tx(&full[s], stage_bytes);
                tma_load_3d(stages + (size_t)s * P.stage_elems, &tmap, boxo[b + STAGES].x, boxo[b + STAGES].y,
                            b + STAGES, &full[s]);
            }
        }
    }

    if (s_abort) {
        // Leave no copy in flight into shared memory this CTA gives back.
        if (tid == 0) {
            const int issued = min(P.N, b + STAGES);
            for (int k = b; k < issued; ++k)
                mbar_wait_bounded(&full[k % STAGES], (uint32_t)(k / STAGES) & 1u, 100000000ull);
        }
        __syncthreads();
        return;
    }

    if (inside) {
        const float fs = P.q_scale ? P.fscale / *P.q_scale : P.fscale;
#pragma unroll
        for (int z = 0; z < TZ; ++z) {
            if (z0 + z < P.nz) {
                float r = 0.f;
                if (active) r = acc[z] * fs;
                float *dst = P.vol + (size_t)(z0 + z) * P.slice_stride + (size_t)y * P.X + x;
                *dst = P.accumulate ? r + *dst : r;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Coefficient-pipeline backprojector.
//
// Every staged tile is expanded once into bilinear coefficients, so that an
// update needs one shared load and four FMAs:
//   FP32 storage:      float4 (Q, dU, dV, dUV)            LDS.128
//   FP16/BF16 storage: uint2  {(Q, dV), (dU, dUV)} pairs   LDS.64 + HFMA2
// The expansion of tile b+1 overlaps the updates of tile b: threads arrive on
// the tile's mbarrier after expanding their share, update from tile b, and
// only then wait for tile b+1, so no CTA-wide barrier stalls the loop.  Three
// coefficient buffers make the reuse safe: a thread may only expand tile b+1
// after passing the wait on tile b, and every thread arrives on tile b only
// after finishing its updates of tile b-2.

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

template <typename S> struct CoefOf;
template <> struct CoefOf<StoreF32> { using E = float4; };
template <> struct CoefOf<StoreF16> { using E = uint2; };
template <> struct CoefOf<StoreBF16> { using E = uint2; };

// FP32 tile [BH][BW] -> float4 coefficients [BH-1][BW] (column BW-1 unused).
// Work item = (quad of columns, band of rows); walking down the band reuses
// the previous raw row.  The fifth column of the last quad is read one
// element past the row (the next row or the stage padding) and only feeds
// the unused last column.
template <int NT>
__device__ __forceinline__ void expand_f32(const float *__restrict__ raw, float4 *__restrict__ coef, int BW, int BH,
                                           int tid)
{
    constexpr int kBand = 4;
    const int nq = BW >> 2;
    const int nrows = BH - 1;
    const int nbands = (nrows + kBand - 1) / kBand;
    for (int item = tid; item < nq * nbands; item += NT) {
        const int cq = item % nq, band = item / nq;
        const int r0 = band * kBand, r1 = min(r0 + kBand, nrows);
        const int c0 = cq << 2;
        float4 a = *reinterpret_cast<const float4 *>(raw + r0 * BW + c0);
        float a4 = raw[r0 * BW + c0 + 4];
        float4 dA = make_float4(a.y - a.x, a.z - a.y, a.w - a.z, a4 - a.w);
        for (int r = r0; r < r1; ++r) {
            const float4 b = *reinterpret_cast<const float4 *>(raw + (r + 1) * BW + c0);
            const float b4 = raw[(r + 1) * BW + c0 + 4];
            const float4 dB = make_float4(b.y - b.x, b.z - b.y, b.w - b.z, b4 - b.w);
            float4 *o = coef + r * BW + c0;
            o[0] = make_float4(a.x, dA.x, b.x - a.x, dB.x - dA.x);
            o[1] = make_float4(a.y, dA.y, b.y - a.y, dB.y - dA.y);
            o[2] = make_float4(a.z, dA.z, b.z - a.z, dB.z - dA.z);
            o[3] = make_float4(a.w, dA.w, b.w - a.w, dB.w - dA.w);
            a = b;
            dA = dB;
        }
    }
}

template <typename S, int NT>
__device__ __forceinline__ void expand_any(const typename S::T *raw, typename CoefOf<S>::E *coef, int BW, int BH,
                                           int tid)
{
    if constexpr (S::kCoef)
        expand_tile<typename S::T, typename Vec2Of<S>::type, NT>(raw, coef, BW, BH, tid);
    else
        expand_f32<NT>(raw, coef, BW, BH, tid);
}

template <typename S, int TZ, bool ALL_IN>
__device__ __forceinline__ void update_column(const typename CoefOf<S>::E *__restrict__ cb, uint32_t cbase, uint32_t BW,
                                              const float (&aZ)[TZ], float (&acc)[TZ], float U, float U2, float fu,
                                              float cZ, float Hm1)
{
    using V2 = typename Vec2Of<S>::type;
    [[maybe_unused]] V2 fu2;
    if constexpr (S::kCoef) fu2 = splat<V2>(fu);
#pragma unroll
    for (int z = 0; z < TZ; ++z) {
        const float v = aZ[z] * U + cZ;
        const float fl = __fadd_rd(v, kMagic);
        const float fv = v - (fl - kMagic);
        const uint32_t o = (uint32_t)__float_as_int(fl) * BW + cbase;
        float A, B;
        if constexpr (S::kCoef) {
            const float2 ab = coef_eval<V2>(cb[o], fu2);
            A = ab.x;
            B = ab.y;
        } else {
            const float4 c = cb[o];
            A = fmaf(fu, c.y, c.x);
            B = fmaf(fu, c.w, c.z);
        }
        const float val = fmaf(fv, B, A);
        if constexpr (ALL_IN) {
            acc[z] = fmaf(U2, val, acc[z]);
        } else {
            const float w = (v >= 0.f && v <= Hm1) ? U2 : 0.f;  // kernel.cu:130-131
            acc[z] = fmaf(w, val, acc[z]);
        }
    }
}

template <typename S, int TX, int TY, int TZ, int RS, int MINB>
__global__ void __launch_bounds__(TX *TY, MINB)
    bp_coef_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ BPParams P)
{
    using T = typename S::T;
    using E = typename CoefOf<S>::E;
    constexpr int NT = TX * TY;
    constexpr int NC = 3;
    extern __shared__ __align__(128) unsigned char smem[];
    T *raw = reinterpret_cast<T *>(smem);
    E *coef = reinterpret_cast<E *>(smem + (size_t)RS * P.stage_elems * sizeof(T));
    int2 *boxo = reinterpret_cast<int2 *>(coef + (size_t)NC * P.coef_stride);
    uint64_t *rfull = reinterpret_cast<uint64_t *>(boxo + P.N);
    uint64_t *cfull = rfull + RS;

    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int x0 = (blockIdx.x % P.tilesX) * TX, y0 = (blockIdx.x / P.tilesX) * TY;
    const int z0 = blockIdx.y * TZ;
    const int x = x0 + tx, y = y0 + ty;
    const float aX = flip(P.scale * ((float)x + P.dX), P.dirx);
    const float aY = flip(P.scale * ((float)y + P.dY), P.diry);
    const bool inside = (x < P.X) && (y < P.Y);
    const bool active = inside && (sqrtf(aX * aX + aY * aY) < P.halfW);

    if (!__syncthreads_or(active)) {  // tile entirely outside the FOV cylinder
        if (inside) {
            for (int z = 0; z < TZ && z0 + z < P.nz; ++z) {
                float *dst = P.vol + (size_t)(z0 + z) * P.slice_stride + (size_t)y * P.X + x;
                *dst = P.accumulate ? 0.f + *dst : 0.f;
            }
        }
        return;
    }

    for (int b = tid; b < P.N; b += NT) boxo[b] = footprint_origin<TX, TY, TZ, S::kAlign>(P, b, x0, y0, z0);
    if (tid == 0) {
        for (int s = 0; s < RS; ++s) mbar_init(&rfull[s], 1);
        for (int k = 0; k < NC; ++k) mbar_init(&cfull[k], NT);
        fence_mbar_init();
        prefetch_tensormap(&tmap);
    }
    __syncthreads();
    const uint32_t stage_bytes = (uint32_t)(P.BW * P.BH * sizeof(T));
    int issued = 0;  // raw tiles requested (meaningful in thread 0)
    auto issue = [&](int tile) {
        const int s = tile % RS;
        mbar_arrive_expect_tx(&rfull[s], stage_bytes);
        tma_load_3d(raw + (size_t)s * P.stage_elems, &tmap, boxo[tile].x, boxo[tile].y, tile, &rfull[s]);
        issued = tile + 1;
    };
    if (tid == 0)
        for (int t = 0; t < RS && t < P.N; ++t) issue(t);

    // Slices past the end of the slab repeat the last one (see the note in
    // bp_tma_kernel): their footprint stays inside the staged box.
    float aZ[TZ];
#pragma unroll
    for (int z = 0; z < TZ; ++z) aZ[z] = flip(P.scale * ((float)min(z0 + z, P.nz - 1) + P.zoff), P.dirz);
    float acc[TZ];
#pragma unroll
    for (int z = 0; z < TZ; ++z) acc[z] = 0.f;

    bool ok = mbar_wait_bounded(&rfull[0], 0u, kWaitLimitNs);
    int consumed = 1;
    if (ok) expand_any<S, NT>(raw, coef, P.BW, P.BH, tid);
    mbar_arrive(&cfull[0]);
    ok = ok && mbar_wait_bounded(&cfull[0], 0u, kWaitLimitNs);
    if (tid == 0 && ok && RS < P.N) issue(RS);

    const float cZ = P.cZ, Hm1 = P.Hm1;
    const uint32_t BW = (uint32_t)P.BW;
    for (int b = 0; b < P.N && ok; ++b) {
        const int nb = b + 1;
        if (nb < P.N) {
            ok = mbar_wait_bounded(&rfull[nb % RS], (uint32_t)(nb / RS) & 1u, kWaitLimitNs);
            consumed = nb + 1;
            if (ok) expand_any<S, NT>(raw + (size_t)(nb % RS) * P.stage_elems, coef + (size_t)(nb % NC) * P.coef_stride,
                                      P.BW, P.BH, tid);
            mbar_arrive(&cfull[nb % NC]);
        }
        if (active && ok) {
            const float2 cs = P.trig[b];
            const float Sd = aX * cs.x + aY * cs.y;
            const float Td = aY * cs.x - aX * cs.y;
            const float U = P.D / (P.D - Sd);
            const float u = Td * U + P.cX;
            if (u >= 0.f && u <= P.Wm1) {  // column inside the detector (kernel.cu:127-128)
                const int bx0 = boxo[b].x, by0 = boxo[b].y;
                const float U2 = U * U;
                const float fla = __fadd_rd(u, kMagic);
                const int col = __float_as_int(fla) - kMagicBits - bx0;
                const float fu = u - (fla - kMagic);
                const float vA = aZ[0] * U + cZ, vB = aZ[TZ - 1] * U + cZ;
                const float vlo = fminf(vA, vB), vhi = fmaxf(vA, vB);
                const int rlo = (int)floorf(vlo) - by0, rhi = (int)floorf(vhi) + 1 - by0;
                if (col >= 0 && col + 1 < P.BW && rlo >= 0 && rhi < P.BH) {
                    const uint32_t cbase = (uint32_t)col - (uint32_t)(kMagicBits + by0) * BW;
                    const E *cb = coef + (size_t)(b % NC) * P.coef_stride;
                    if (vlo >= 0.f && vhi <= Hm1)
                        update_column<S, TZ, true>(cb, cbase, BW, aZ, acc, U, U2, fu, cZ, Hm1);
                    else
                        update_column<S, TZ, false>(cb, cbase, BW, aZ, acc, U, U2, fu, cZ, Hm1);
                } else {
                    atomicOr(P.err, ERR_BOX_OVERFLOW);
                }
            }
        }
        if (nb < P.N && ok) {
            ok = mbar_wait_bounded(&cfull[nb % NC], (uint32_t)(nb / NC) & 1u, kWaitLimitNs);
            // every thread has expanded tile nb: its raw stage is free again
            if (tid == 0 && ok && nb + RS < P.N) issue(nb + RS);
        }
    }

    if (!ok) {
        atomicOr(P.err, ERR_WAIT_TIMEOUT);
        // Leave no copy in flight into shared memory this CTA gives back.
        if (tid == 0)
            for (int k = consumed; k < issued; ++k)
                mbar_wait_bounded(&rfull[k % RS], (uint32_t)(k / RS) & 1u, 100000000ull);
        return;
    }

    if (inside) {
        const float fs = P.q_scale ? P.fscale / *P.q_scale : P.fscale;
#pragma unroll
        for (int z = 0; z < TZ; ++z) {
            if (z0 + z < P.nz) {
                float r = 0.f;
                if (active) r = acc[z] * fs;
                float *dst = P.vol + (size_t)(z0 + z) * P.slice_stride + (size_t)y * P.X + x;
                *dst = P.accumulate ? r + *dst : r;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// host side

static PFN_cuTensorMapEncodeTiled_v12000 get_encode_fn()
{
    static PFN_cuTensorMapEncodeTiled_v12000 fn = nullptr;
    if (!fn) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            fn = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    return fn;
}

struct BPVariant {
    const void *fn;
    int precision, TX, TY, TZ, STAGES;
    bool coef;  // coefficient pipeline (bp_coef_kernel) or direct FP32 gathers (bp_tma_kernel)
    const char *name;
};

#define TK_BP_DIRECT(S, P, TX, TY, TZ, ST, MB) \
    {reinterpret_cast<const void *>(&bp_tma_kernel<S, TX, TY, TZ, ST, MB>), P, TX, TY, TZ, ST, false, \
     "direct<" #S "," #TX "," #TY "," #TZ "," #ST ">"}
#define TK_BP_COEF(S, P, TX, TY, TZ, ST, MB) \
    {reinterpret_cast<const void *>(&bp_coef_kernel<S, TX, TY, TZ, ST, MB>), P, TX, TY, TZ, ST, true, \
     "coef<" #S "," #TX "," #TY "," #TZ "," #ST ">"}

// The first entry of each precision is the default.
static const BPVariant kVariants[] = {
    TK_BP_COEF(StoreF32, TK_F32, 16, 16, 32, 3, 2),
    TK_BP_COEF(StoreF16, TK_F16, 16, 16, 32, 3, 2),
    TK_BP_COEF(StoreBF16, TK_BF16, 16, 16, 32, 3, 2),
    TK_BP_DIRECT(StoreF32, TK_F32, 16, 16, 32, 4, 2),
    TK_BP_DIRECT(StoreF16, TK_F16, 16, 16, 32, 4, 2),
};

static int g_variant_override = -1;  // index into kVariants, set by tk_bp_select_variant

static const BPVariant *pick_variant(int precision)
{
    if (g_variant_override >= 0 && kVariants[g_variant_override].precision == precision)
        return &kVariants[g_variant_override];
    for (const auto &v : kVariants)
        if (v.precision == precision) return &v;
    return nullptr;
}

// Analytic bound of a tile's footprint extent (see the derivation in the
// design notes): for two voxels of one tile,
//   |du| <= s*dxy*Umax + Rmax*D/(D-Rmax)^2*s*dxy,
//   |dv| <= s*(TZ-1)*Umax + |aZ|max*D/(D-Rmax)^2*s*dxy.
static int box_dims(const tk_geometry &g, int nz, float zoff, const BPVariant &v, int align, int *BW, int *BH)
{
    const double s = std::fabs((double)g.scale), D = g.D;
    const double ex = s * std::fmax(std::fabs(0.0 - g.cx), std::fabs((double)(g.X - 1) - g.cx)) + 1.0;
    const double ey = s * std::fmax(std::fabs(0.0 - g.cy), std::fabs((double)(g.Y - 1) - g.cy)) + 1.0;
    const double R = std::sqrt(ex * ex + ey * ey);
    TK_CHECK(D - R > 1e-3 * D, TK_ERR_UNSUPPORTED,
             "volume corners (radius %.1f px) reach the source (D = %.1f px)", R, D);
    const double Umax = D / (D - R), dU = D / ((D - R) * (D - R));
    const double dxy = s * std::sqrt((double)(v.TX - 1) * (v.TX - 1) + (double)(v.TY - 1) * (v.TY - 1));
    const double azmax = s * std::fmax(std::fabs((double)zoff), std::fabs((double)(nz - 1) + zoff)) + 1.0;
    const double du = dxy * Umax + R * dU * dxy;
    const double dv = s * (v.TZ - 1) * Umax + azmax * dU * dxy;
    int bw = (int)std::floor(du) + 9 + align;
    bw = (bw + align - 1) / align * align;
    int bh = (int)std::floor(dv) + 7;
    TK_CHECK(bw <= 256 && bh <= 256, TK_ERR_UNSUPPORTED,
             "tile footprint %dx%d exceeds the 256x256 TMA box", bw, bh);
    *BW = bw;
    *BH = bh;
    return TK_OK;
}

int launch_backproject(const tk_geometry &g, const void *d_q, int precision, const float *d_q_scale, int nz,
                       float zoff, float *d_vol, int accumulate, cudaStream_t stream)
{
    if (int rc = validate_geometry(&g)) return rc;
    TK_CHECK(d_q && d_vol, TK_ERR_INVALID, "backproject: null device pointer");
    TK_CHECK(nz >= 0, TK_ERR_INVALID, "backproject: nz < 0");
    TK_CHECK(precision == TK_F32 || d_q_scale, TK_ERR_INVALID, "backproject: 16-bit storage needs its scale");
    if (nz == 0) return TK_OK;
    const BPVariant *v = pick_variant(precision);
    TK_CHECK(v, TK_ERR_INVALID, "backproject: unknown precision %d", precision);
    auto encode = get_encode_fn();
    TK_CHECK(encode, TK_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");

    const int align = precision == TK_F32 ? 4 : 8;
    int BW, BH;
    if (int rc = box_dims(g, nz, zoff, *v, align, &BW, &BH)) return rc;

    std::vector<float> cs(g.N), sn(g.N);
    build_trig(g, cs.data(), sn.data());
    const int p = reference_pad_length(g.W);

    const int tilesX = (g.X + v->TX - 1) / v->TX, tilesY = (g.Y + v->TY - 1) / v->TY;
    const int zchunks = (nz + v->TZ - 1) / v->TZ;
    TK_CHECK((long long)tilesX * tilesY < (1ll << 31) && zchunks < 65536, TK_ERR_UNSUPPORTED,
             "volume too large for one launch");

    const size_t esz = elem_size(precision);
    const int Wp = row_pitch(g.W);
    static thread_local BPParams P;  // ~26 KB: keep off the stack
    std::memset(&P, 0, sizeof(P));
    P.err = device_error_word();
    TK_CHECK(P.err, TK_ERR_CUDA, "device error word unavailable");
    P.vol = d_vol;
    P.slice_stride = (long long)g.X * g.Y;
    P.X = g.X;
    P.Y = g.Y;
    P.nz = nz;
    P.BW = BW;
    P.BH = BH;
    P.stage_elems = (BW * BH + 63) / 64 * 64;  // 128-byte aligned stages for any element size
    P.coef_stride = (BW * (BH - 1) + 15) / 16 * 16;
    P.tilesX = tilesX;
    P.accumulate = accumulate ? 1 : 0;
    P.cX = g.cX;
    P.cZ = g.cZ;
    P.D = g.D;
    P.dX = -g.cx;
    P.dY = -g.cy;
    P.zoff = zoff;
    P.scale = g.scale;
    P.dirx = g.dirx ? 0x80000000u : 0u;
    P.diry = g.diry ? 0x80000000u : 0u;
    P.dirz = g.dirz ? 0x80000000u : 0u;
    P.Wm1 = (float)(g.W - 1);
    P.Hm1 = (float)(g.H - 1);
    P.halfW = g.W / 2.;
    // result *= delta_f * scaling, with scaling = 1/p (kernel.cu:113, 575)
    P.fscale = g.dfi * (1.f / (float)p);
    P.q_scale = d_q_scale;

    for (int b0 = 0; b0 < g.N; b0 += kMaxParamProj) {
        const int nb = std::min(kMaxParamProj, g.N - b0);
        P.N = nb;
        for (int b = 0; b < nb; ++b) P.trig[b] = make_float2(cs[b0 + b], sn[b0 + b]);
        P.accumulate = (accumulate || b0 > 0) ? 1 : 0;

        CUtensorMap tmap;
        const char *base = static_cast<const char *>(d_q) + (size_t)b0 * g.H * Wp * esz;
        cuuint64_t dims[3] = {(cuuint64_t)g.W, (cuuint64_t)g.H, (cuuint64_t)nb};
        cuuint64_t strides[2] = {(cuuint64_t)Wp * esz, (cuuint64_t)Wp * g.H * esz};
        cuuint32_t box[3] = {(cuuint32_t)BW, (cuuint32_t)BH, 1};
        cuuint32_t estr[3] = {1, 1, 1};
        CUtensorMapDataType dt = precision == TK_F32   ? CU_TENSOR_MAP_DATA_TYPE_FLOAT32
                                 : precision == TK_F16 ? CU_TENSOR_MAP_DATA_TYPE_FLOAT16
                                                       : CU_TENSOR_MAP_DATA_TYPE_BFLOAT16;
        CUresult cr = encode(&tmap, dt, 3, const_cast<char *>(base), dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        TK_CHECK(cr == CUDA_SUCCESS, TK_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)cr);

        size_t smem = (size_t)v->STAGES * P.stage_elems * esz;
        if (v->coef)
            smem += 3 * (size_t)P.coef_stride * (precision == TK_F32 ? sizeof(float4) : sizeof(uint2));
        else if (precision != TK_F32)
            smem += 2 * (size_t)P.coef_stride * sizeof(uint2);
        smem += (size_t)nb * sizeof(int2) + (size_t)(v->STAGES + 3) * sizeof(uint64_t) + 16;
        TK_CHECK(smem <= 227 * 1024, TK_ERR_UNSUPPORTED, "backproject: %zu B of shared memory needed", smem);
        TK_CUDA(cudaFuncSetAttribute(v->fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        dim3 grid((unsigned)(tilesX * tilesY), (unsigned)zchunks, 1);
        dim3 block((unsigned)(v->TX * v->TY), 1, 1);
        void *args[] = {&tmap, &P};
        TK_CUDA(cudaLaunchKernel(v->fn, grid, block, args, smem, stream));
    }
    return TK_OK;
}

}  // namespace tk

// ---------------------------------------------------------------------------
// variant selection (benchmarking and the autotuner)

extern "C" int tk_bp_variant_count(void) { return (int)(sizeof(tk::kVariants) / sizeof(tk::kVariants[0])); }

extern "C" const char *tk_bp_variant_name(int i)
{
    if (i < 0 || i >= tk_bp_variant_count()) return "";
    return tk::kVariants[i].name;
}

extern "C" int tk_bp_variant_precision(int i)
{
    if (i < 0 || i >= tk_bp_variant_count()) return -1;
    return tk::kVariants[i].precision;
}

extern "C" int tk_bp_select_variant(int i)
{
    if (i < -1 || i >= tk_bp_variant_count()) {
        tk::set_error("no backprojection variant %d", i);
        return TK_ERR_INVALID;
    }
    tk::g_variant_override = i;
    return TK_OK;
}
