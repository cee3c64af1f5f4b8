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
#include "tk_bp_core.cuh"
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
    int tilesX, tilesY;
    int accumulate;
    float cX, cZ, D;
    float dX, dY, zoff, scale;
    unsigned dirx, diry, dirz;  // 0 or 0x80000000 (sign flip, kernel.cu:86-88)
    float Wm1, Hm1;             // W-1, H-1
    float halfW;                // W / 2. (kernel.cu:100 compares in double; W / 2 is exact in FP32, as is
                                // the sqrtf result, so the FP32 comparison decides the same)
    float fscale;               // dfi * (1/p)  (kernel.cu:113)
    const float *q_scale;       // device storage scale of the filtered projections, or null (= 1)
    int qbase, qlen;  // quarter-turn kernel: steps q = qbase + (t mod qlen) + (t / qlen) N/4, t < 4 qlen
    int qf0, qfs;     // ... and the image frame of q + k N/4: qf0 + (q - qbase) mod N/4 + quarter * qfs
    float2 trig[kMaxParamProj]; // (cos, sin) per projection (kernel.cu:430-441)
};

// Storage traits -------------------------------------------------------------
struct StoreF32 {
    using T = float;
    static constexpr int kAlign = 4;  // TMA x coordinate granularity (16 B)
    static constexpr bool kCoef = false;
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

// Bilinear interpolation and weighted accumulation of two voxels with packed
// FP32: per lane exactly top = fma(fu, q01-q00, q00), bot = fma(fu, q11-q10,
// q10), acc = fma(w, fma(fv, bot-top, top), acc).
__device__ __forceinline__ void bilinear_acc_x2(float q00a, float q00b, float q01a, float q01b, float q10a,
                                                float q10b, float q11a, float q11b, float fu, float fva, float fvb,
                                                float wa, float wb, float &acc0, float &acc1)
{
    asm("{\n\t.reg .b64 Q00, Q01, Q10, Q11, FU, FV, W, C, D0, D1;\n\t"
        "mov.b64 Q00, {%2, %3};\n\t"
        "mov.b64 Q01, {%4, %5};\n\t"
        "mov.b64 Q10, {%6, %7};\n\t"
        "mov.b64 Q11, {%8, %9};\n\t"
        "mov.b64 FU, {%10, %10};\n\t"
        "mov.b64 FV, {%11, %12};\n\t"
        "mov.b64 W, {%13, %14};\n\t"
        "mov.b64 C, {%0, %1};\n\t"
        "sub.rn.f32x2 D0, Q01, Q00;\n\t"
        "sub.rn.f32x2 D1, Q11, Q10;\n\t"
        "fma.rn.f32x2 Q00, FU, D0, Q00;\n\t"
        "fma.rn.f32x2 Q10, FU, D1, Q10;\n\t"
        "sub.rn.f32x2 D0, Q10, Q00;\n\t"
        "fma.rn.f32x2 Q00, FV, D0, Q00;\n\t"
        "fma.rn.f32x2 C, W, Q00, C;\n\t"
        "mov.b64 {%0, %1}, C;\n\t}"
        : "+f"(acc0), "+f"(acc1)
        : "f"(q00a), "f"(q00b), "f"(q01a), "f"(q01b), "f"(q10a), "f"(q10b), "f"(q11a), "f"(q11b), "f"(fu),
          "f"(fva), "f"(fvb), "f"(wa), "f"(wb));
}

// One column's update of the direct kernel over its TZ slices; PACKED walks
// two slices per step with packed FP32 and gives the same bits.
template <int TZ, bool ALL_IN, bool PACKED>
__device__ __forceinline__ void direct_update(const float *st, uint32_t BW, uint32_t cbase, float fu, float U,
                                              float U2, float cZ, float Hm1, const float (&aZ)[TZ], float (&acc)[TZ])
{
    if constexpr (PACKED && (TZ % 2 == 0)) {
#pragma unroll
        for (int z = 0; z < TZ; z += 2) {
            const float va = slice_v(aZ[z], U, cZ), vb = slice_v(aZ[z + 1], U, cZ);
            float fla, flb, fva, fvb;
            floor_frac_x2(va, vb, fla, flb, fva, fvb);
            const uint32_t oa = (uint32_t)__float_as_int(fla) * BW + cbase;
            const uint32_t ob = (uint32_t)__float_as_int(flb) * BW + cbase;
            float wa = U2, wb = U2;
            if constexpr (!ALL_IN) {
                wa = (va >= 0.f && va <= Hm1) ? U2 : 0.f;  // kernel.cu:130-131
                wb = (vb >= 0.f && vb <= Hm1) ? U2 : 0.f;
            }
            bilinear_acc_x2(st[oa], st[ob], st[oa + 1], st[ob + 1], st[oa + BW], st[ob + BW], st[oa + BW + 1],
                            st[ob + BW + 1], fu, fva, fvb, wa, wb, acc[z], acc[z + 1]);
        }
    } else {
#pragma unroll
        for (int z = 0; z < TZ; ++z) {
            const float v = slice_v(aZ[z], U, cZ);
            const float fl = __fadd_rd(v, kMagic);
            const float fv = v - (fl - kMagic);
            const uint32_t o = (uint32_t)__float_as_int(fl) * BW + cbase;
            const float q00 = st[o], q01 = st[o + 1];
            const float q10 = st[o + BW], q11 = st[o + BW + 1];
            const float top = fmaf(fu, q01 - q00, q00);
            const float bot = fmaf(fu, q11 - q10, q10);
            const float w = ALL_IN ? U2 : ((v >= 0.f && v <= Hm1) ? U2 : 0.f);  // kernel.cu:130-131
            acc[z] = fmaf(w, fmaf(fv, bot - top, top), acc[z]);
        }
    }
}

// ---------------------------------------------------------------------------
// Direct FP32 backprojector: bilinear gathers straight from the staged
// sample tile (four LDS.32 per update).
template <typename S, int TX, int TY, int TZ, int STAGES, int MINB, bool PACKED = false>
__global__ void __launch_bounds__(TX *TY, MINB)
    bp_tma_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ BPParams P)
{
    using T = typename S::T;
    static_assert(sizeof(T) == 4, "direct kernel: FP32 samples only");
    constexpr int NT = TX * TY;
    extern __shared__ __align__(128) unsigned char smem[];

    T *stages = reinterpret_cast<T *>(smem);
    int2 *boxo = reinterpret_cast<int2 *>(smem + (size_t)STAGES * P.stage_elems * sizeof(T));
    uint64_t *full = reinterpret_cast<uint64_t *>(boxo + P.N);
    volatile int &s_abort = *reinterpret_cast<int *>(full + STAGES);

    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int2 tile = tile_of(blockIdx.x, P.tilesX, P.tilesY);
    const int x0 = tile.x * TX, y0 = tile.y * TY;
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
        if (active && got) {
            float U, u;
            column_geometry(aX, aY, P.trig[b], P.D, P.cX, U, u);
            if (u >= 0.f && u <= P.Wm1) {  // column inside the detector (kernel.cu:127-128)
                const float U2 = __fmul_rn(U, U);
                const float fla = __fadd_rd(u, kMagic);
                const int a = __float_as_int(fla) - kMagicBits;
                const float fu = u - (fla - kMagic);
                const int col = a - bx0;
                const float vA = slice_v(aZ[0], U, cZ), vB = slice_v(aZ[TZ - 1], U, cZ);
                const float vlo = fminf(vA, vB), vhi = fmaxf(vA, vB);
                const int rlo = (int)floorf(vlo) - by0, rhi = (int)floorf(vhi) + 1 - by0;
                if (col >= 0 && col + 1 < P.BW && rlo >= 0 && rhi < P.BH) {
                    const uint32_t cbase = (uint32_t)col - (uint32_t)(kMagicBits + by0) * BW;
                    const bool all_in = (vlo >= 0.f) && (vhi <= Hm1);
                    const float *st = reinterpret_cast<const float *>(stages) + (size_t)s * P.stage_elems;
                    if (all_in)
                        direct_update<TZ, true, PACKED>(st, BW, cbase, fu, U, U2, cZ, Hm1, aZ, acc);
                    else
                        direct_update<TZ, false, PACKED>(st, BW, cbase, fu, U, U2, cZ, Hm1, aZ, acc);
                } else {
                    atomicOr(P.err, ERR_BOX_OVERFLOW);
                }
            }
        }
        __syncthreads();  // every thread is done with stage s
        if (s_abort) break;
        if (tid == 0 && b + STAGES < P.N) {
            mbar_arrive_expect_tx(&full[s], stage_bytes);
            tma_load_3d(stages + (size_t)s * P.stage_elems, &tmap, boxo[b + STAGES].x, boxo[b + STAGES].y,
                        b + STAGES, &full[s]);
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
// Coefficient-image backprojector.
//
// The filter writes each projection as an image of bilinear coefficient
// entries (see tk_precision): entry (r, c) covers the detector cell
// [r, r+1] x [c, c+1], so an update is one shared load of one entry and
//   A = Q + fu dU,  B = dV + fu dUV,  acc += U^2 (A + fv B)
// (FP16/BF16: A and B come from one packed HFMA2).  The staged box holds
// entries, one row/column smaller than a sample box.  v is walked linearly,
// v_z = v0 + z dv with dv = scale * U, which frees the per-slice registers
// for a 64-voxel z column.  Loads use 32-bit shared addresses (inline PTX)
// so the address of an update is one IMAD.

// Bounding-box origin (entries) of a tile's footprint; the z range is
// [z0, z1] in slab slices.
template <int TX, int TY, int ALIGN>
__device__ __forceinline__ int2 footprint_origin_z(const BPParams &P, int b, int x0, int y0, int z0, int z1)
{
    const float2 cs = P.trig[b];
    const int xs[2] = {x0, min(x0 + TX - 1, P.X - 1)};
    const int ys[2] = {y0, min(y0 + TY - 1, P.Y - 1)};
    const float aZ0 = flip(P.scale * ((float)z0 + P.zoff), P.dirz);
    const float aZ1 = flip(P.scale * ((float)z1 + P.zoff), P.dirz);
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
            vmin = fminf(vmin, fminf(aZ0 * U + P.cZ, aZ1 * U + P.cZ));
        }
    }
    int bx = (int)floorf(umin) - 1;
    bx &= ~(ALIGN - 1);
    return make_int2(bx, (int)floorf(vmin) - 1);
}

template <int PREC, int TX, int TY, int TZ, int STAGES, bool PARTIAL, int MINB, int WALK = 0>
__global__ void __launch_bounds__(TX *TY, MINB)
    bp_cimg_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ BPParams P)
{
    constexpr int NT = TX * TY;
    constexpr int ES = Cimg<PREC>::kBytes;
    extern __shared__ __align__(128) unsigned char smem[];
    int2 *boxo = reinterpret_cast<int2 *>(smem + (size_t)STAGES * P.stage_elems * ES);
    uint64_t *full = reinterpret_cast<uint64_t *>(boxo + P.N);
    volatile int &s_abort = *reinterpret_cast<int *>(full + STAGES);

    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const int2 tile = tile_of(blockIdx.x, P.tilesX, P.tilesY);
    const int x0 = tile.x * TX, y0 = tile.y * TY;
    // Full chunks of TZ slices.  16-bit storage: the last chunk, when fewer than
    // TZ slices are left, walks only those slices (always with PARTIAL, for
    // nz < TZ).  FP32 coefficients (the plain form, TZ | nz at the sizes it is
    // timed on): the last chunk is moved down to end at nz and stores only the
    // slices no earlier chunk owns, which keeps its walk free of the runtime choice.
    const int zc = blockIdx.y * TZ;
    constexpr bool kRuntimeRagged = PREC != TK_F32_COEF;
    const bool ragged = PARTIAL || (kRuntimeRagged && zc + TZ > P.nz);
    const int z0 = (PARTIAL || kRuntimeRagged) ? zc : min(zc, P.nz - TZ);
    const int zlast = ragged ? P.nz - 1 - z0 : TZ - 1;
    const int x = x0 + tx, y = y0 + ty;
    const float aX = flip(P.scale * ((float)x + P.dX), P.dirx);
    const float aY = flip(P.scale * ((float)y + P.dY), P.diry);
    const bool inside = (x < P.X) && (y < P.Y);
    const bool active = inside && (sqrtf(aX * aX + aY * aY) < P.halfW);

    if (!__syncthreads_or(active)) {  // tile entirely outside the FOV cylinder
        if (inside) {
            for (int z = max(zc - z0, 0); z <= zlast; ++z) {
                float *dst = P.vol + (size_t)(z0 + z) * P.slice_stride + (size_t)y * P.X + x;
                *dst = P.accumulate ? 0.f + *dst : 0.f;
            }
        }
        return;
    }

    for (int b = tid; b < P.N; b += NT) boxo[b] = footprint_origin_z<TX, TY, Cimg<PREC>::kAlign>(P, b, x0, y0, z0, z0 + zlast);
    if (tid == 0) {
        s_abort = 0;
        for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
        prefetch_tensormap(&tmap);
    }
    __syncthreads();
    const uint32_t stage_bytes = (uint32_t)(P.BW * P.BH * ES);
    const uint32_t smem0 = smem_u32(smem);
    // the tensor map's innermost dimension counts floats: ES/4 per entry
    if (tid == 0) {
        for (int s = 0; s < STAGES && s < P.N; ++s) {
            mbar_arrive_expect_tx(&full[s], stage_bytes);
            tma_load_3d(smem + (size_t)s * P.stage_elems * ES, &tmap, boxo[s].x * (ES / 4), boxo[s].y, s, &full[s]);
        }
    }

    const float aZ0 = flip(P.scale * ((float)z0 + P.zoff), P.dirz);
    const float daZ = flip(P.scale, P.dirz);
    float acc[TZ];
#pragma unroll
    for (int z = 0; z < TZ; ++z) acc[z] = 0.f;

    const float cZ = P.cZ, Hm1 = P.Hm1;
    const uint32_t row_bytes = (uint32_t)P.BW * ES;
    int b = 0;
    for (; b < P.N; ++b) {
        const int s = b % STAGES;
        const uint32_t parity = (uint32_t)(b / STAGES) & 1u;
        const bool got = mbar_wait_bounded(&full[s], parity, kWaitLimitNs);
        if (!got) {
            atomicOr(P.err, ERR_WAIT_TIMEOUT);
            s_abort = 1;
        }
        if (active && got) {
            float U, u;
            column_geometry(aX, aY, P.trig[b], P.D, P.cX, U, u);
            if (u >= 0.f && u <= P.Wm1) {  // column inside the detector (kernel.cu:127-128)
                const int bx0 = boxo[b].x, by0 = boxo[b].y;
                const float fla = __fadd_rd(u, kMagic);
                const int col = __float_as_int(fla) - kMagicBits - bx0;
                const float fu = u - (fla - kMagic);
                const float v0 = slice_v(aZ0, U, cZ);
                const float dv = __fmul_rn(daZ, U);
                const float vL = fmaf((float)zlast, dv, v0);
                const float vlo = fminf(v0, vL), vhi = fmaxf(v0, vL);
                const int rlo = (int)floorf(vlo) - by0, rhi = (int)floorf(vhi) - by0;
                if (col >= 0 && col < P.BW && rlo >= 0 && rhi < P.BH) {
                    const uint32_t sbase = smem0 + (uint32_t)s * P.stage_elems * ES + (uint32_t)col * ES -
                                           (uint32_t)(kMagicBits + by0) * row_bytes;
                    const float U2 = __fmul_rn(U, U);
                    if (vlo >= 0.f && vhi <= Hm1)
                        if (ragged)
                            update_cimg<PREC, TZ, true, true, WALK>(sbase, row_bytes, v0, dv, fu, U2, Hm1, zlast, acc);
                        else
                            update_cimg<PREC, TZ, true, false, WALK>(sbase, row_bytes, v0, dv, fu, U2, Hm1, zlast,
                                                                      acc);
                    else
                        if (ragged)
                            update_cimg<PREC, TZ, false, true, WALK>(sbase, row_bytes, v0, dv, fu, U2, Hm1, zlast,
                                                                      acc);
                        else
                            update_cimg<PREC, TZ, false, false, WALK>(sbase, row_bytes, v0, dv, fu, U2, Hm1, zlast,
                                                                       acc);
                } else {
                    atomicOr(P.err, ERR_BOX_OVERFLOW);
                }
            }
        }
        __syncthreads();  // every thread is done with stage s
        if (s_abort) break;
        if (tid == 0 && b + STAGES < P.N) {
            mbar_arrive_expect_tx(&full[s], stage_bytes);
            tma_load_3d(smem + (size_t)s * P.stage_elems * ES, &tmap, boxo[b + STAGES].x * (ES / 4),
                        boxo[b + STAGES].y, b + STAGES, &full[s]);
        }
    }

    if (s_abort) {
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
            if (z <= zlast && z0 + z >= zc) {
                float r = 0.f;
                if (active) r = acc[z] * fs;
                float *dst = P.vol + (size_t)(z0 + z) * P.slice_stride + (size_t)y * P.X + x;
                *dst = P.accumulate ? r + *dst : r;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// The quarter-turn kernel's walk of one step: a column's 16 slices at four
// projections a quarter turn apart, whose entries sit at the same offsets in
// the step's four boxes (sbase + k CAPB).  fu, U^2 and the row coordinates
// v_z = fma(z, dv, v0) are shared by the four.  Past the chunk's last slice
// (a partial chunk ending on an even slice) the pair's second slice repeats
// the first, whose rows are inside the box, at weight 0.
template <int PREC, int INTERP, int CAPB, bool PARTIAL, int ROWI, int TZ>
__device__ __forceinline__ void quad_walk(uint32_t sbase, uint32_t row_bytes, float v0, float dv, float fu, float U2,
                                          float Hm1, bool all_in, int zlast, float (&acc)[4][TZ])
{
    if constexpr (PREC == TK_F32_COEF) {
        // shared-memory bound (a 16-byte load per voxel): no software pipeline
#pragma unroll
        for (int z = 0; z < TZ; z += 2) {
            if (PARTIAL && z > zlast) break;
            const bool bin = !PARTIAL || z + 1 <= zlast;
            const float va = fmaf((float)z, dv, v0);
            const float vb = bin ? fmaf((float)(z + 1), dv, v0) : va;
            float fla, flb, fva, fvb;
            floor_frac_x2(va, vb, fla, flb, fva, fvb);
            const uint32_t ra = (uint32_t)__float_as_int(fla) * row_bytes + sbase;
            const uint32_t rb = (uint32_t)__float_as_int(flb) * row_bytes + sbase;
            float wa = U2, wb = bin ? U2 : 0.f;
            if (!all_in) {  // kernel.cu:130-131
                wa = (va >= 0.f && va <= Hm1) ? wa : 0.f;
                wb = (vb >= 0.f && vb <= Hm1) ? wb : 0.f;
            }
            float e[4][8];
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                             : "=f"(e[k][0]), "=f"(e[k][1]), "=f"(e[k][2]), "=f"(e[k][3])
                             : "r"(ra + (uint32_t)(k * CAPB)));
                asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];"
                             : "=f"(e[k][4]), "=f"(e[k][5]), "=f"(e[k][6]), "=f"(e[k][7])
                             : "r"(rb + (uint32_t)(k * CAPB)));
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {  // entry (Q, dU, dV, dUV)
                const float Aa = fmaf(fu, e[k][1], e[k][0]), Ba = fmaf(fu, e[k][3], e[k][2]);
                const float Ab = fmaf(fu, e[k][5], e[k][4]), Bb = fmaf(fu, e[k][7], e[k][6]);
                acc[k][z] = fmaf(wa, fmaf(fva, Ba, Aa), acc[k][z]);
                if (!PARTIAL || z + 1 < TZ) acc[k][z + 1] = fmaf(wb, fmaf(fvb, Bb, Ab), acc[k][z + 1]);
            }
        }
    } else {
        // 8-byte entries {(Q, dV), (dU, dUV)}, software-pipelined: pair p+1's coordinates,
        // fractions and eight loads are issued before pair p's arithmetic
        uint32_t e[2][4][4];  // [buffer][k][lo a, hi a, lo b, hi b]
        float fvp[2][2], wp[2][2];
        uint32_t fvh[2], wh[2];
        const __half2 U2h2 = __float2half2_rn(U2);
        const uint32_t w_all = *reinterpret_cast<const uint32_t *>(&U2h2);
        auto fetch = [&](int z, int bi) {
            const bool bin = !PARTIAL || z + 1 <= zlast;
            const float va = fmaf((float)z, dv, v0);
            const float vb = bin ? fmaf((float)(z + 1), dv, v0) : va;
            float fla, flb, fva, fvb;
            floor_frac_x2(va, vb, fla, flb, fva, fvb);
            const uint32_t ra = (uint32_t)__float_as_int(fla) * row_bytes + sbase;
            const uint32_t rb = (uint32_t)__float_as_int(flb) * row_bytes + sbase;
            const bool ina = all_in || (va >= 0.f && va <= Hm1);  // kernel.cu:130-131
            const bool inb = bin && (all_in || (vb >= 0.f && vb <= Hm1));
            if constexpr (INTERP == 1) {
                fvp[bi][0] = fva;
                fvp[bi][1] = fvb;
                wp[bi][0] = ina ? U2 : 0.f;
                wp[bi][1] = inb ? U2 : 0.f;
            } else {
                const __half2 f2 = __floats2half2_rn(fva, fvb);
                fvh[bi] = *reinterpret_cast<const uint32_t *>(&f2);
                wh[bi] = (ina ? (w_all & 0xffffu) : 0u) | (inb ? (w_all & 0xffff0000u) : 0u);
            }
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];"
                             : "=r"(e[bi][k][0]), "=r"(e[bi][k][1])
                             : "r"(ra + (uint32_t)(k * CAPB)));
                asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];"
                             : "=r"(e[bi][k][2]), "=r"(e[bi][k][3])
                             : "r"(rb + (uint32_t)(k * CAPB)));
            }
        };
        const __half2 fuh = __float2half2_rn(fu);
        fetch(0, 0);
#pragma unroll
        for (int z = 0; z < TZ; z += 2) {
            if (PARTIAL && z > zlast) break;
            const int bi = (z / 2) & 1;
            if (z + 2 < TZ && (!PARTIAL || z + 2 <= zlast)) fetch(z + 2, bi ^ 1);
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                if constexpr (INTERP == 1 && PREC == TK_F16) {
                    // scalar FMAs: 2 % faster than the f32x2 form for FP16, 6 % slower for BF16
                    interp_scalar_acc<PREC>(e[bi][k][0], e[bi][k][1], e[bi][k][2], e[bi][k][3], fu, fvp[bi][0],
                                            fvp[bi][1], wp[bi][0], wp[bi][1], acc[k][z], acc[k][z + 1]);
                } else if constexpr (INTERP == 1) {
                    float qa, dva, dua, duva, qb, dvb, dub, duvb;
                    unpack_pair<PREC>(e[bi][k][0], qa, dva);
                    unpack_pair<PREC>(e[bi][k][1], dua, duva);
                    unpack_pair<PREC>(e[bi][k][2], qb, dvb);
                    unpack_pair<PREC>(e[bi][k][3], dub, duvb);
                    interp4_acc_x2(qa, qb, dua, dub, dva, dvb, duva, duvb, fu, fvp[bi][0], fvp[bi][1], wp[bi][0],
                                   wp[bi][1], acc[k][z], acc[k][z + 1]);
                } else {
                    const __half2 ha = __hfma2(*reinterpret_cast<const __half2 *>(&e[bi][k][1]), fuh,
                                               *reinterpret_cast<const __half2 *>(&e[bi][k][0]));
                    const __half2 hb = __hfma2(*reinterpret_cast<const __half2 *>(&e[bi][k][3]), fuh,
                                               *reinterpret_cast<const __half2 *>(&e[bi][k][2]));
                    if (ROWI == 0) {
                        const __half2 val = __hfma2(*reinterpret_cast<const __half2 *>(&fvh[bi]),
                                                    __highs2half2(ha, hb), __lows2half2(ha, hb));
                        acc_mixed_x2(*reinterpret_cast<const uint32_t *>(&val), wh[bi], acc[k][z], acc[k][z + 1]);
                    } else {
                        row_acc_x2(*reinterpret_cast<const uint32_t *>(&ha), *reinterpret_cast<const uint32_t *>(&hb),
                                   fvh[bi], wh[bi], acc[k][z], acc[k][z + 1]);
                    }
                }
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Quarter-turn backprojector (coefficient images): a circular scan of a
// square, centred, unflipped volume maps onto itself under a quarter turn.
// Voxel column (x, y) at angle beta and the column R(x, y) = (X-1-y, x) at
// beta + 90 degrees have the same S, T, U and u (S' = -aY (-sin) + aX cos = S,
// T' = aX (-sin) + aY cos = T), so one column geometry, one row coordinate
// and one floor / fraction / address per slice pair serve four
// (column, projection) pairs: column c of tile T at projection q and its
// turns R^k(c) at projection (q + k N/4) mod N.  A CTA owns one orbit
// {T, R(T), R^2(T), R^3(T)} of 16 x TYQ-column tiles (T in the first
// quadrant) and 16 slices, and steps through the projections q of an angle
// set closed under quarter turns (all N, or the quarter-turn images of one
// range [qbase, qbase + qlen)); over the steps each of the four columns sees
// every projection of the set once.  Step q stages four boxes at T's
// footprint origin in projection q (projections (q + k N/4) mod N), one TMA
// load each on one mbarrier, in slots of CAPB bytes (immediate load offsets).
// Used when the host has checked that the tabulated angles (q + k N/4) mod N
// are within 1e-5 rad of beta_q + k pi/2.
//
// Storage and arithmetic (PREC, INTERP):
//   TK_F16 / TK_BF16, INTERP 1 (the default): per slice pair and turn k, two
//     LDS.64 (the pair's entries), the eight 16-bit values converted exactly
//     to FP32, then FP32 interpolation and accumulation (FP16: scalar FMAs,
//     interp_scalar_acc; BF16: four fma.rn.f32x2, interp4_acc_x2): per voxel
//     the operations of update_cimg's walk 4;
//   TK_F16, INTERP 0 (selectable half-math form): update_cimg's walk 3 --
//     column interpolation by HFMA2, row interpolation by one FP16 FMA, U^2
//     rounded to FP16 and applied by fma.rn.f32.f16;
//   TK_F32_COEF, INTERP 1: one LDS.128 per voxel and the same FP32
//     operations as scalar FMAs.
// The 8-byte forms are software-pipelined: pair p+1's coordinates, fractions
// and eight loads are issued before pair p's arithmetic.
template <int PREC, int INTERP, int CAPB, int STAGES, bool PARTIAL, int ROWI, int ISSUE, int GEO = 0, int TYQ = 16,
          int TZQ = 16>
__global__ void __launch_bounds__(16 * TYQ, (PREC == TK_F32_COEF ? 2 : 32 / TYQ))
    bp_quad_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ BPParams P)
{
    // tiles of 16 x TYQ columns (TYQ 16: 2 CTAs of 8 warps per SM; TYQ 8: 4 CTAs of 4 warps)
    constexpr int TX = 16, TY = TYQ, TZ = TZQ, NT = TX * TY, ES = Cimg<PREC>::kBytes;
    static_assert(ISSUE == 0 || NT / 32 >= 4, "four issuing warps");
    static_assert(INTERP == 1 || PREC == TK_F16, "the half-math walk is FP16 only");
    extern __shared__ __align__(128) unsigned char smem[];
    const int NQ = P.N / 4;  // a quarter turn in projections
    const int steps = 4 * P.qlen;
    // footprint origins as 16-bit pairs (the host keeps W, H below 2^14): 4 qlen <= 3200 steps in 12.8 KB
    short2 *boxo = reinterpret_cast<short2 *>(smem + (size_t)STAGES * 4 * CAPB);
    uint64_t *full = reinterpret_cast<uint64_t *>(boxo + steps);  // steps = 4 qlen: 8-byte aligned
    auto qof = [&](int t) { return P.qbase + t % P.qlen + (t / P.qlen) * NQ; };
    volatile int &s_abort = *reinterpret_cast<volatile int *>(full + STAGES);
    int *s_issued = reinterpret_cast<int *>(full + STAGES) + 1;  // steps issued so far

    const int tid = threadIdx.x;
    const int lx = tid % TX, ly = tid / TX;
    const int2 tile = tile_of(blockIdx.x, P.tilesX / 2, P.tilesY / 2);  // a tile of the first quadrant
    const int x0 = tile.x * TX, y0 = tile.y * TY;
    const int zc = blockIdx.y * TZ;
    const int z0 = PARTIAL ? zc : min(zc, P.nz - TZ);
    const int zlast = PARTIAL ? P.nz - 1 - z0 : TZ - 1;
    const int x = x0 + lx, y = y0 + ly;
    const float aX = P.scale * ((float)x + P.dX);
    const float aY = P.scale * ((float)y + P.dY);
    const bool active = sqrtf(aX * aX + aY * aY) < P.halfW;  // the same for the four turned columns
    const int Xm1 = P.X - 1;
    // column R^k(x, y) as a volume offset
    const size_t colk[4] = {(size_t)y * P.X + x, (size_t)x * P.X + (Xm1 - y), (size_t)(Xm1 - y) * P.X + (Xm1 - x),
                            (size_t)(Xm1 - x) * P.X + y};

    if (!__syncthreads_or(active)) {  // the orbit lies outside the FOV cylinder
        for (int z = max(zc - z0, 0); z <= zlast; ++z)
            for (int k = 0; k < 4; ++k) {
                float *dst = P.vol + (size_t)(z0 + z) * P.slice_stride + colk[k];
                *dst = P.accumulate ? 0.f + *dst : 0.f;
            }
        return;
    }

    for (int t = tid; t < steps; t += NT) {
        const int2 o = footprint_origin_z<TX, TY, Cimg<PREC>::kAlign>(P, qof(t), x0, y0, z0, z0 + zlast);
        boxo[t] = make_short2((short)o.x, (short)o.y);
    }
    if (tid == 0) {
        s_abort = 0;
        *s_issued = min(steps, STAGES);
        for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], ISSUE == 0 ? 1 : 4);
        fence_mbar_init();
        prefetch_tensormap(&tmap);
    }
    __syncthreads();
    const uint32_t box_bytes = (uint32_t)(P.BW * P.BH * ES);
    const uint32_t smem0 = smem_u32(smem);
    // ISSUE 0: thread 0 issues a step's four boxes; ISSUE 1: lane 0 of warp k < 4 issues box k
    // (one arrival with its bytes each, so the stage completes with the fourth), which spreads
    // the refill's delay after each step's barrier over four warps.
    const int wid = tid >> 5;
    const bool issuer = ISSUE == 0 ? tid == 0 : ((tid & 31) == 0 && wid < 4);
    // step t = kk qlen + r is projection q = qbase + r + kk N/4; its k-th box comes from projection
    // (q + k N/4) mod N, image frame qf0 + r + ((kk + k) mod 4) qfs (the whole image: qf0 = qbase,
    // qfs = N/4; a compact image of the four ranges: qf0 = 0, qfs = qlen)
    int ri = 0, kki = 0;  // the issuer's (r, kk) of the next step to issue, kept by increments
    auto issue = [&](int t, int s) {  // the boxes of step t into stage s
        const int r = ri, kk = kki;
        if (++ri == P.qlen) {
            ri = 0;
            ++kki;
        }
        const short2 bo = boxo[t];
        if (ISSUE == 0) {
            mbar_arrive_expect_tx(&full[s], 4 * box_bytes);
            for (int k = 0; k < 4; ++k) {
                const int f = P.qf0 + r + ((kk + k) & 3) * P.qfs;
                tma_load_3d(smem + (size_t)(s * 4 + k) * CAPB, &tmap, bo.x * (ES / 4), bo.y, f, &full[s]);
            }
        } else {
            const int f = P.qf0 + r + ((kk + wid) & 3) * P.qfs;
            mbar_arrive_expect_tx(&full[s], box_bytes);
            tma_load_3d(smem + (size_t)(s * 4 + wid) * CAPB, &tmap, bo.x * (ES / 4), bo.y, f, &full[s]);
        }
    };
    if (issuer)
        for (int s = 0; s < STAGES && s < steps; ++s) issue(s, s);

    const float aZ0 = flip(P.scale * ((float)z0 + P.zoff), P.dirz);
    const float daZ = flip(P.scale, P.dirz);
    float acc[4][TZ];
#pragma unroll
    for (int k = 0; k < 4; ++k)
#pragma unroll
        for (int z = 0; z < TZ; ++z) acc[k][z] = 0.f;

    const float cZ = P.cZ, Hm1 = P.Hm1;
    const uint32_t row_bytes = (uint32_t)P.BW * ES;
    // A CTA barrier ends each step, then the issuing warps refill the stage.  (Releasing stages
    // per warp instead, with the last warp done refilling, measured 7 % slower.)  GEO 1: the
    // step's column geometry (a divide and the trig load) is formed before the stage's wait.
    int t = 0;
    int qt = P.qbase, rt = 0;  // qof(t), kept by increments: t mod qlen in rt
    for (; t < steps; ++t) {
        const int s = t % STAGES;
        const uint32_t parity = (uint32_t)(t / STAGES) & 1u;
        float Ue = 0.f, ue = 0.f;
        if constexpr (GEO == 1) column_geometry(aX, aY, P.trig[qt], P.D, P.cX, Ue, ue);  // before the wait
        const bool got = mbar_wait_bounded(&full[s], parity, kWaitLimitNs);
        if (!got) {
            atomicOr(P.err, ERR_WAIT_TIMEOUT);
            s_abort = 1;
        }
        if (got && active) {
            float U = Ue, u = ue;
            if constexpr (GEO == 0) column_geometry(aX, aY, P.trig[qt], P.D, P.cX, U, u);
            if (u >= 0.f && u <= P.Wm1) {  // column inside the detector (kernel.cu:127-128)
                const int bx0 = boxo[t].x, by0 = boxo[t].y;
                const float fla = __fadd_rd(u, kMagic);
                const int col = __float_as_int(fla) - kMagicBits - bx0;
                const float fu = u - (fla - kMagic);
                const float v0 = slice_v(aZ0, U, cZ);
                const float dv = __fmul_rn(daZ, U);
                const float vL = fmaf((float)zlast, dv, v0);
                const float vlo = fminf(v0, vL), vhi = fmaxf(v0, vL);
                const int rlo = (int)floorf(vlo) - by0, rhi = (int)floorf(vhi) - by0;
                if (col >= 0 && col < P.BW && rlo >= 0 && rhi < P.BH) {
                    const uint32_t sbase = smem0 + (uint32_t)(s * 4) * CAPB + (uint32_t)col * ES -
                                           (uint32_t)(kMagicBits + by0) * row_bytes;
                    const float U2 = __fmul_rn(U, U);
                    const bool all_in = vlo >= 0.f && vhi <= Hm1;
                    quad_walk<PREC, INTERP, CAPB, PARTIAL, ROWI, TZ>(sbase, row_bytes, v0, dv, fu, U2, Hm1, all_in,
                                                                zlast, acc);
                } else {
                    atomicOr(P.err, ERR_BOX_OVERFLOW);
                }
            }
        }
        __syncthreads();  // every thread is done with stage s
        if (s_abort) break;
        if (issuer && t + STAGES < steps) {
            issue(t + STAGES, s);
            if (tid == 0) *s_issued = t + STAGES + 1;
        }
        if (++rt == P.qlen) {
            rt = 0;
            qt += NQ - P.qlen + 1;
        } else {
            ++qt;
        }
    }

    if (s_abort) {  // (every thread left the loop at the same step, after the barrier)
        const int issued = *s_issued;
        if (tid == 0)  // the copies in flight land before the CTA's shared memory is released
            for (int k = max(0, issued - STAGES); k < issued; ++k)
                mbar_wait_bounded(&full[k % STAGES], (uint32_t)(k / STAGES) & 1u, 100000000ull);
        __syncthreads();
        return;
    }

    const float fs = P.q_scale ? P.fscale / *P.q_scale : P.fscale;
#pragma unroll
    for (int z = 0; z < TZ; ++z) {
        if (z <= zlast && z0 + z >= zc) {
#pragma unroll
            for (int k = 0; k < 4; ++k) {
                const float r = active ? acc[k][z] * fs : 0.f;
                float *dst = P.vol + (size_t)(z0 + z) * P.slice_stride + colk[k];
                *dst = P.accumulate ? r + *dst : r;
            }
        }
    }
}

// ---------------------------------------------------------------------------
// Forward projector: the exact transpose of the bilinear backprojector
// (bp_tma_kernel, the FP32-sample storage that tk_fdk_forward uses).
//
// For every voxel v in the FOV, projection b and voxel value g[v], the
// backprojection reads q_b at (u, v') with bilinear weights and adds
// fscale * U^2 * interp to the voxel; the transpose adds
// fscale * U^2 * g[v] * weight to each of the four samples.  Masks are the
// same: u in [0, W-1], v' in [0, H-1] (kernel.cu:127-131), FOV (kernel.cu:100).
// A CTA scatters its voxel tile's contributions for one projection into a
// shared-memory box with shared atomics, then adds the box to the global
// gradient with one TMA reduce (cp.reduce.async.bulk.tensor ... .add).
// Conflicts: in a warp the lanes that share a detector column would hit the
// same cell at every z (rays along x put all 16 x-lanes on one column), so
// lane l handles slice (k + l) mod 32 at step k; lanes then sit on different
// rows, and the accumulation box has an odd row pitch (BW + 1) so that
// different rows of one column fall in different banks.  After the atomics
// the box is drained into one of two dense staging boxes (the TMA source,
// pitch BW) and cleared in the same pass; a staging box is rewritten only
// after the reduce that read it.  Reduces never start at a negative
// coordinate: the box origin is clamped to >= 0, which only drops samples
// outside the detector (weight 0 anyway).
template <int TX, int TY, bool PARTIAL>
__global__ void __launch_bounds__(TX *TY, 2)
    fp_scatter_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ BPParams P,
                      const float *__restrict__ vin)
{
    constexpr int NT = TX * TY;
    constexpr int TZ = 32;  // one slice per lane of a warp at every step
    extern __shared__ __align__(128) unsigned char smem[];
    const int BW = P.BW, BWp = P.BW + 1, BH = P.BH;
    float *staging = reinterpret_cast<float *>(smem);           // 2 x [BH][BW]
    float *acc = staging + 2 * (size_t)P.stage_elems;            // [BH][BW + 1]
    int2 *boxo = reinterpret_cast<int2 *>(acc + (size_t)((BH * BWp + 31) & ~31));

    const int tid = threadIdx.x, lane = tid & 31;
    const int tx = tid % TX, ty = tid / TX;
    const int2 tile = tile_of(blockIdx.x, P.tilesX, P.tilesY);
    const int x0 = tile.x * TX, y0 = tile.y * TY;
    const int zc = blockIdx.y * TZ;
    const int z0 = PARTIAL ? zc : min(zc, P.nz - TZ);
    const int zlast = PARTIAL ? P.nz - 1 - z0 : TZ - 1;
    const int x = x0 + tx, y = y0 + ty;
    const float aX = flip(P.scale * ((float)x + P.dX), P.dirx);
    const float aY = flip(P.scale * ((float)y + P.dY), P.diry);
    const bool inside = (x < P.X) && (y < P.Y);
    const bool active = inside && (sqrtf(aX * aX + aY * aY) < P.halfW);
    if (!__syncthreads_or(active)) return;  // nothing in this tile projects

    for (int b = tid; b < P.N; b += NT) {
        int2 o = footprint_origin_z<TX, TY, 4>(P, b, x0, y0, z0, z0 + zlast);
        o.x = max(o.x, 0);  // still a multiple of 4
        o.y = max(o.y, 0);
        boxo[b] = o;
    }
    for (int i = tid; i < BH * BWp; i += NT) acc[i] = 0.f;
    // This thread's voxel values (scaled) and slice coordinates in its
    // rotated slice order; slices owned by another chunk, or past the end,
    // carry 0.  aZ is formed per voxel exactly as bp_tma_kernel forms it, so
    // the masks v in [0, H-1] agree voxel by voxel and this is the transpose
    // of that kernel to FP32 rounding of the weights.
    float g[TZ], aZ[TZ];
#pragma unroll
    for (int k = 0; k < TZ; ++k) {
        const int z = (k + lane) & (TZ - 1);
        g[k] = 0.f;
        if (active && z <= zlast && z0 + z >= zc)
            g[k] = P.fscale * vin[(size_t)(z0 + z) * P.slice_stride + (size_t)y * P.X + x];
        aZ[k] = flip(P.scale * ((float)min(z0 + z, P.nz - 1) + P.zoff), P.dirz);
    }
    const float aZf = flip(P.scale * ((float)z0 + P.zoff), P.dirz);
    const float aZl = flip(P.scale * ((float)(z0 + zlast) + P.zoff), P.dirz);
    const float cZ = P.cZ, Hm1 = P.Hm1;
    __syncthreads();

    for (int b = 0; b < P.N; ++b) {
        const int bx0 = boxo[b].x, by0 = boxo[b].y;
        if (active) {
            float U, u;
            column_geometry(aX, aY, P.trig[b], P.D, P.cX, U, u);
            if (u >= 0.f && u <= P.Wm1) {
                const float fla = __fadd_rd(u, kMagic);
                const int col = __float_as_int(fla) - kMagicBits - bx0;
                const float fu = u - (fla - kMagic);
                const float U2 = __fmul_rn(U, U);
                const float v0 = slice_v(aZf, U, cZ), vL = slice_v(aZl, U, cZ);
                const float vlo = fmaxf(fminf(v0, vL), 0.f), vhi = fminf(fmaxf(v0, vL), Hm1);
                if (vlo <= vhi) {
                    const int rlo = (int)floorf(vlo) - by0, rhi = (int)floorf(vhi) + 1 - by0;
                    if (col >= 0 && col + 1 < BW && rlo >= 0 && rhi < BH) {
                        float *base = acc + col;
#pragma unroll
                        for (int k = 0; k < TZ; ++k) {
                            const float v = slice_v(aZ[k], U, cZ);
                            if (g[k] != 0.f && v >= 0.f && v <= Hm1) {
                                const float fl = __fadd_rd(v, kMagic);
                                const float fv = v - (fl - kMagic);
                                const int row = __float_as_int(fl) - kMagicBits - by0;
                                const float w = U2 * g[k];
                                const float w1 = w * fu, w0 = w - w1;  // columns col, col+1
                                float *r0 = base + row * BWp;
                                atomicAdd(r0, w0 - w0 * fv);
                                atomicAdd(r0 + 1, w1 - w1 * fv);
                                atomicAdd(r0 + BWp, w0 * fv);
                                atomicAdd(r0 + BWp + 1, w1 * fv);
                            }
                        }
                    } else {
                        atomicOr(P.err, ERR_BOX_OVERFLOW);
                    }
                }
            }
        }
        float *st = staging + (size_t)(b & 1) * P.stage_elems;
        if (tid == 0 && b >= 2) bulk_wait_group_read<1>();  // the reduce of b-2 has read this staging box
        __syncthreads();
        for (int i = tid; i < BH * BW; i += NT) {
            const int r = i / BW, c = i - r * BW;
            float *a = acc + r * BWp + c;
            st[i] = *a;
            *a = 0.f;
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            if (bx0 < (int)P.Wm1 + 1 && by0 < (int)P.Hm1 + 1) tma_reduce_add_3d(&tmap, bx0, by0, b, st);
            bulk_commit_group();  // one group per projection, empty when the box misses the detector
        }
    }
    if (tid == 0) bulk_wait_group_all();
}

// ---------------------------------------------------------------------------
// Forward projector with slice lanes (the default form; same weights, masks,
// box and drain as fp_scatter_kernel).  Lane l of warp w holds slice z0 + l
// of the warp's 32 voxel columns (tile rows 2w and 2w+1), and the warp walks
// its columns one by one.  The lanes of one shared atomic then sit on the
// rows of 32 consecutive slices of one column: distinct rows whenever the
// row step |scale| U is at least one, and with the odd row pitch (BW + 1)
// distinct banks for rows less than 32 apart.  The column geometry of a
// projection is computed once per column (lane j for column j) into a
// per-warp table in shared memory and read back as a broadcast.
//
// FIXED: the box accumulates two-word fixed point with native integer shared
// atomics instead of FP32 shared atomics (an FP32 add to shared memory is a
// load and compare-and-swap loop).  Each CTA scales its contributions by a
// power of two s chosen from the tile's largest possible contribution
// max|g| U^2_max, so that each scaled contribution c has |c| <= 2^hb,
// hb = min(30 - cbits, 22), where at most 2^cbits <= 2^13 contributions reach
// one cell of one projection (bound formed on the host from the row step and
// the ray strip).  c is split exactly into round(c) (the hi word) and the
// remainder c - round(c), |.| <= 1/2 (<= 1 where rounding lifts |c| a few
// ulps past 2^22), which is rounded to 2^-kb units (kb = hb; the lo word).
// Neither word's cell sum can pass 2^30, the integer sums are exact, and the
// resolution is 2^-(hb + kb) of the tile's largest contribution (2^-34 or
// finer) against FP32 atomics' rounding of every partial sum.  The drain
// forms (hi + lo 2^-kb) / s in FP32.  For finite inputs.
// FIXED 2 (cbits <= 9) drops the hi word's bias subtraction: the bits of
// c + 1.5 2^23 are 0x4B400000 + round(c), and 0x4B400000 is a multiple of
// 2^22, so the low 22 bits of a cell's sum of raw bits are its sum of round(c)
// modulo 2^22, exact while that sum stays inside +-2^21 (hb = 20 - cbits); the
// drain sign-extends them.  The lo word keeps its subtraction, with
// kb = min(22, 30 - cbits): resolution 2^-(hb + kb), 2^-32 or finer.
// FIXED 3 (cbits <= 8) windows the lo word the same way (kb = 21 - cbits, its
// cell sums also inside +-2^20): no subtraction at all, resolution 2^-25 or
// finer.  FIXED 1 takes both subtractions (any cbits <= 13); 0 the FP32 atomics.
template <int TX, int TY, bool PARTIAL, int FIXED = 0>
__global__ void __launch_bounds__(TX *TY, 2)
    fp_scatter_col_kernel(const __grid_constant__ CUtensorMap tmap, const __grid_constant__ BPParams P,
                          const float *__restrict__ vin, float u2max, int cbits)
{
    constexpr int NT = TX * TY, NW = NT / 32, TZ = 32;
    static_assert(TX == 16 && NT == 256, "a warp owns two tile rows of 16 columns");
    extern __shared__ __align__(128) unsigned char smem[];
    const int BW = P.BW, BWp = P.BW + 1, BH = P.BH;
    float *staging = reinterpret_cast<float *>(smem);  // 2 x [BH][BW]
    float *acc = staging + 2 * (size_t)P.stage_elems;   // [BH][BW + 1] (FIXED: hi words, then lo words)
    const int acc_elems = (BH * BWp + 31) & ~31;
    int *acc_hi = reinterpret_cast<int *>(acc), *acc_lo = acc_hi + acc_elems;
    float4 *geo = reinterpret_cast<float4 *>(acc + (FIXED ? 2 : 1) * acc_elems);  // [NW][32] (U, fu, col, U^2)
    int2 *boxo = reinterpret_cast<int2 *>(geo + NW * 32);
    __shared__ float s_gmax[NW];

    const int tid = threadIdx.x, lane = tid & 31, w = tid >> 5;
    const int2 tile = tile_of(blockIdx.x, P.tilesX, P.tilesY);
    const int x0 = tile.x * TX, y0 = tile.y * TY;
    const int zc = blockIdx.y * TZ;
    const int z0 = PARTIAL ? zc : min(zc, P.nz - TZ);
    const int zlast = PARTIAL ? P.nz - 1 - z0 : TZ - 1;
    // column `lane` of this warp, for the geometry of each projection
    const int gx = x0 + (lane & 15), gy = y0 + 2 * w + (lane >> 4);
    const float gaX = flip(P.scale * ((float)gx + P.dX), P.dirx);
    const float gaY = flip(P.scale * ((float)gy + P.dY), P.diry);
    const bool gactive = (gx < P.X) && (gy < P.Y) && (sqrtf(gaX * gaX + gaY * gaY) < P.halfW);
    if (!__syncthreads_or(gactive)) return;  // nothing in this tile projects

    for (int b = tid; b < P.N; b += NT) {
        int2 o = footprint_origin_z<TX, TY, 4>(P, b, x0, y0, z0, z0 + zlast);
        o.x = max(o.x, 0);  // still a multiple of 4
        o.y = max(o.y, 0);
        boxo[b] = o;
    }
    for (int i = tid; i < BH * BWp; i += NT) acc[i] = 0.f;
    if constexpr (FIXED)
        for (int i = tid; i < BH * BWp; i += NT) acc_lo[i] = 0;
    // this lane's slice of the warp's 32 columns (0 for slices owned by another chunk or past the end)
    const unsigned act = __ballot_sync(0xffffffffu, gactive);
    const bool zown = lane <= zlast && z0 + lane >= zc;
    float g[32];
#pragma unroll
    for (int j = 0; j < 32; ++j) {
        const int x = x0 + (j & 15), y = y0 + 2 * w + (j >> 4);
        g[j] = 0.f;
        if (((act >> j) & 1u) && zown)
            g[j] = P.fscale * vin[(size_t)(z0 + lane) * P.slice_stride + (size_t)y * P.X + x];
    }
    if constexpr (FIXED) {
        float m = 0.f;
#pragma unroll
        for (int j = 0; j < 32; ++j) m = fmaxf(m, fabsf(g[j]));
        for (int o = 16; o > 0; o >>= 1) m = fmaxf(m, __shfl_xor_sync(0xffffffffu, m, o));
        if (lane == 0) s_gmax[w] = m;
    }
    const float aZ = flip(P.scale * ((float)min(z0 + lane, P.nz - 1) + P.zoff), P.dirz);
    const float aZf = flip(P.scale * ((float)z0 + P.zoff), P.dirz);
    const float aZl = flip(P.scale * ((float)(z0 + zlast) + P.zoff), P.dirz);
    const float cZ = P.cZ, Hm1 = P.Hm1;
    float4 *gw = geo + w * 32;
    __syncthreads();
    float fx_inv = 1.f, lo_scale = 1.f, lo_unit = 1.f;  // FIXED: 1/s, 2^kb, 2^-kb
    if constexpr (FIXED) {
        float m = 0.f;
#pragma unroll
        for (int k = 0; k < NW; ++k) m = fmaxf(m, s_gmax[k]);
        const float cmax = m * u2max;
        const int hb = FIXED >= 2 ? 20 - cbits : min(30 - cbits, 22);
        const int kb = FIXED == 3 ? 21 - cbits : FIXED == 2 ? min(22, 30 - cbits) : hb;
        int e = 0;
        if (cmax > 0.f && cmax <= 3.0e38f) {
            int ex;
            (void)frexpf(cmax, &ex);  // cmax < 2^ex
            e = max(-126, min(126, hb - ex));
        }
        const float fx_s = ldexpf(1.f, e);
        fx_inv = ldexpf(1.f, -e);
        lo_scale = ldexpf(1.f, kb);
        lo_unit = ldexpf(1.f, -kb);
#pragma unroll
        for (int j = 0; j < 32; ++j) g[j] *= fx_s;
    }

    for (int b = 0; b < P.N; ++b) {
        const int bx0 = boxo[b].x, by0 = boxo[b].y;
        {
            float4 e = make_float4(0.f, 0.f, __int_as_float(-1), 0.f);  // col -1: nothing to scatter
            if (gactive) {
                float U, u;
                column_geometry(gaX, gaY, P.trig[b], P.D, P.cX, U, u);
                if (u >= 0.f && u <= P.Wm1) {
                    const float fla = __fadd_rd(u, kMagic);
                    const int col = __float_as_int(fla) - kMagicBits - bx0;
                    const float fu = u - (fla - kMagic);
                    const float v0 = slice_v(aZf, U, cZ), vL = slice_v(aZl, U, cZ);
                    const float vlo = fmaxf(fminf(v0, vL), 0.f), vhi = fminf(fmaxf(v0, vL), Hm1);
                    if (vlo <= vhi) {
                        const int rlo = (int)floorf(vlo) - by0, rhi = (int)floorf(vhi) + 1 - by0;
                        if (col >= 0 && col + 1 < BW && rlo >= 0 && rhi < BH)
                            e = make_float4(U, fu, __int_as_float(col), __fmul_rn(U, U));
                        else
                            atomicOr(P.err, ERR_BOX_OVERFLOW);
                    }
                }
            }
            gw[lane] = e;
        }
        __syncwarp();
#pragma unroll
        for (int j = 0; j < 32; ++j) {
            const float4 e = gw[j];  // the same entry for every lane
            const int col = __float_as_int(e.z);
            if (col >= 0) {
                const float v = slice_v(aZ, e.x, cZ);
                if (g[j] != 0.f && v >= 0.f && v <= Hm1) {
                    const float fl = __fadd_rd(v, kMagic);
                    const float fv = v - (fl - kMagic);
                    const int row = __float_as_int(fl) - kMagicBits - by0;
                    const float wt = e.w * g[j];
                    const float w1 = wt * e.y, w0 = wt - w1;  // columns col, col+1
                    const int o = row * BWp + col;
                    if constexpr (FIXED) {
                        // c = round(c) + r exactly (|c| <= 2^22: adding 1.5 2^23 rounds to an integer);
                        // the words take round(c) and round(r 2^kb)
                        auto put = [&](int k, float c) {
                            const float hm = __fadd_rn(c, kMagic);
                            const float r = __fsub_rn(c, __fsub_rn(hm, kMagic));
                            const float lm = __fmaf_rn(r, lo_scale, kMagic);
                            if constexpr (FIXED >= 2)
                                atomicAdd(reinterpret_cast<unsigned *>(acc_hi) + k, __float_as_uint(hm));
                            else
                                atomicAdd(acc_hi + k, __float_as_int(hm) - kMagicBits);
                            if constexpr (FIXED == 3)
                                atomicAdd(reinterpret_cast<unsigned *>(acc_lo) + k, __float_as_uint(lm));
                            else
                                atomicAdd(acc_lo + k, __float_as_int(lm) - kMagicBits);
                        };
                        put(o, w0 - w0 * fv);
                        put(o + 1, w1 - w1 * fv);
                        put(o + BWp, w0 * fv);
                        put(o + BWp + 1, w1 * fv);
                    } else {
                        float *r0 = acc + o;
                        atomicAdd(r0, w0 - w0 * fv);
                        atomicAdd(r0 + 1, w1 - w1 * fv);
                        atomicAdd(r0 + BWp, w0 * fv);
                        atomicAdd(r0 + BWp + 1, w1 * fv);
                    }
                }
            }
        }
        float *st = staging + (size_t)(b & 1) * P.stage_elems;
        if (tid == 0 && b >= 2) bulk_wait_group_read<1>();  // the reduce of b-2 has read this staging box
        __syncthreads();  // also: every warp is done with its geometry table
        for (int i = tid; i < BH * BW; i += NT) {
            const int r = i / BW, c = i - r * BW;
            const int k = r * BWp + c;
            if constexpr (FIXED) {
                const int hs = FIXED >= 2 ? (int)((unsigned)acc_hi[k] << 10) >> 10 : acc_hi[k];
                const int ls = FIXED == 3 ? (int)((unsigned)acc_lo[k] << 10) >> 10 : acc_lo[k];
                st[i] = fmaf((float)ls, lo_unit, (float)hs) * fx_inv;
                acc_hi[k] = 0;
                acc_lo[k] = 0;
            } else {
                st[i] = acc[k];
                acc[k] = 0.f;
            }
        }
        fence_proxy_async_smem();
        __syncthreads();
        if (tid == 0) {
            if (bx0 < (int)P.Wm1 + 1 && by0 < (int)P.Hm1 + 1) tma_reduce_add_3d(&tmap, bx0, by0, b, st);
            bulk_commit_group();  // one group per projection, empty when the box misses the detector
        }
    }
    if (tid == 0) bulk_wait_group_all();
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
    const void *fn_partial;  // nz < TZ (coefficient kernels only)
    int precision, TX, TY, TZ, STAGES;
    bool coef;  // coefficient image (bp_cimg_kernel) or raw FP32 samples (bp_tma_kernel)
    const char *name;
    int qcap = 0;  // > 0: bp_quad_kernel with staged boxes of up to qcap bytes (needs quad_eligible)
    bool qauto = false;  // a quarter-turn variant the default selection tries, in table order
};


#define TK_BP_DIRECT(TX, TY, TZ, ST) \
    {reinterpret_cast<const void *>(&bp_tma_kernel<StoreF32, TX, TY, TZ, ST, 2>), nullptr, TK_F32, TX, TY, TZ, ST, \
     false, "direct<f32," #TX "," #TY "," #TZ "," #ST ">"}
#define TK_BP_DIRECT_PK(TX, TY, TZ, ST) \
    {reinterpret_cast<const void *>(&bp_tma_kernel<StoreF32, TX, TY, TZ, ST, 2, true>), nullptr, TK_F32, TX, TY, TZ, \
     ST, false, "direct_x2<f32," #TX "," #TY "," #TZ "," #ST ">"}
#define TK_BP_CIMG(P, PN, TX, TY, TZ, ST, MB) \
    {reinterpret_cast<const void *>(&bp_cimg_kernel<P, TX, TY, TZ, ST, false, MB>), \
     reinterpret_cast<const void *>(&bp_cimg_kernel<P, TX, TY, TZ, ST, true, MB>), P, TX, TY, TZ, ST, true, \
     "cimg<" PN "," #TX "," #TY "," #TZ "," #ST ",occ" #MB ">"}

#define TK_BP_CIMG_PK(P, PN, TX, TY, TZ, ST, MB) \
    {reinterpret_cast<const void *>(&bp_cimg_kernel<P, TX, TY, TZ, ST, false, MB, 1>), \
     reinterpret_cast<const void *>(&bp_cimg_kernel<P, TX, TY, TZ, ST, true, MB, 1>), P, TX, TY, TZ, ST, true, \
     "cimg_x2<" PN "," #TX "," #TY "," #TZ "," #ST ",occ" #MB ">"}
// quarter-turn kernels, for symmetric scans only: PREC storage, INTERP 1 FP32 interpolation
// (update_cimg walk 4's operations), INTERP 0 the FP16 half-math walk 3 (ROWI 1) or 2 (ROWI 0)
#define TK_BP_QUAD_TZ(P, PN, IN, INAME, CAP, ST, ROWI, ISSUE, AUTO, GEO, TY, TZ) \
    {reinterpret_cast<const void *>(&bp_quad_kernel<P, IN, CAP, ST, false, ROWI, ISSUE, GEO, TY, TZ>), \
     reinterpret_cast<const void *>(&bp_quad_kernel<P, IN, CAP, ST, true, ROWI, ISSUE, GEO, TY, TZ>), P, 16, TY, TZ, \
     ST, true, "quad<" PN ",16," #TY "," #TZ "," #ST ",cap" #CAP "," INAME ",issue" #ISSUE ",geo" #GEO ">", CAP, AUTO}
#define TK_BP_QUAD_T(P, PN, IN, INAME, CAP, ST, ROWI, ISSUE, AUTO, GEO, TY) \
    TK_BP_QUAD_TZ(P, PN, IN, INAME, CAP, ST, ROWI, ISSUE, AUTO, GEO, TY, 16)
#define TK_BP_QUADF(P, PN, CAP, ST, AUTO, TY) TK_BP_QUAD_T(P, PN, 1, "f32i", CAP, ST, 1, 1, AUTO, 1, TY)
#define TK_BP_QUADH(CAP, ST, ROWI, ISSUE, AUTO, GEO, TY) \
    TK_BP_QUAD_T(TK_F16, "f16", 0, "h16row" #ROWI, CAP, ST, ROWI, ISSUE, AUTO, GEO, TY)
// FP16 half-math walks (update_cimg WALK 2 and 3, same bits): not bit-identical to the FP32 walks
#define TK_BP_CIMG_H2(TX, TY, TZ, ST, MB, WK) \
    {reinterpret_cast<const void *>(&bp_cimg_kernel<TK_F16, TX, TY, TZ, ST, false, MB, WK>), \
     reinterpret_cast<const void *>(&bp_cimg_kernel<TK_F16, TX, TY, TZ, ST, true, MB, WK>), TK_F16, TX, TY, TZ, ST, \
     true, "cimg_h" #WK "<f16," #TX "," #TY "," #TZ "," #ST ",occ" #MB ">"}
// 16-bit storage with FP32 interpolation (update_cimg WALK 4)
#define TK_BP_CIMG_F(P, PN, TX, TY, TZ, ST, MB) \
    {reinterpret_cast<const void *>(&bp_cimg_kernel<P, TX, TY, TZ, ST, false, MB, 4>), \
     reinterpret_cast<const void *>(&bp_cimg_kernel<P, TX, TY, TZ, ST, true, MB, 4>), P, TX, TY, TZ, ST, true, \
     "cimg_f32i<" PN "," #TX "," #TY "," #TZ "," #ST ",occ" #MB ">"}

// The first entry of each storage format is its default.  Every default
// interpolates in FP32 (FP32 geometry, interpolation weights, interpolation and
// accumulation; 16-bit storage converted exactly to FP32).  Where a format has
// automatic quarter-turn variants (FP16 and BF16) its first entry is one; the automatic quarter-turn
// alternatives (qauto, in table order) take larger footprints, and a scan
// without the symmetry runs the format's first general entry.  FP16 storage:
// the quarter-turn kernel with 16 x 8 tiles, else walk 4.  The half-math
// walks (FP16 interpolation arithmetic) are selectable only.
static const BPVariant kVariants[] = {
    TK_BP_DIRECT_PK(16, 16, 32, 4),
    TK_BP_QUADF(TK_F16, "f16", 6144, 2, true, 8),
    TK_BP_CIMG_F(TK_F16, "f16", 16, 16, 64, 3, 2),
    TK_BP_QUADF(TK_BF16, "bf16", 6144, 2, true, 8),
    TK_BP_CIMG_F(TK_BF16, "bf16", 16, 16, 64, 3, 2),
    TK_BP_CIMG_PK(TK_F32_COEF, "f32c", 16, 16, 64, 2, 2),
    TK_BP_DIRECT(16, 16, 32, 4),
    TK_BP_QUADF(TK_F16, "f16", 8192, 2, true, 16),   // 16 x 16 tiles when a 16 x 8 tile's footprint exceeds 6 KB
    TK_BP_QUADF(TK_F16, "f16", 13824, 2, true, 16),  // footprints of up to 13.5 KB (scales near 1.5)
    TK_BP_QUADF(TK_BF16, "bf16", 8192, 2, true, 16),
    TK_BP_QUADF(TK_BF16, "bf16", 13824, 2, true, 16),
    // FP32 coefficients by quarter turns (selectable): 16 bytes of shared memory per voxel update keep
    // it at the shared-memory bandwidth, where it runs slower than the general walk above
    TK_BP_QUADF(TK_F32_COEF, "f32c", 13312, 2, false, 16),
    TK_BP_QUADH(6144, 2, 1, 1, false, 1, 8),  // the FP16 half-math forms
    TK_BP_QUADH(8192, 2, 1, 1, false, 1, 16),
    TK_BP_QUADH(13824, 2, 1, 1, false, 1, 16),
    TK_BP_QUADH(8192, 3, 1, 0, false, 0, 16),
    TK_BP_QUADH(8192, 3, 0, 0, false, 0, 16),
    TK_BP_CIMG_H2(16, 16, 64, 3, 2, 3),
    TK_BP_CIMG_H2(16, 16, 64, 3, 2, 2),
    TK_BP_CIMG_PK(TK_F16, "f16", 16, 16, 64, 3, 2),
    TK_BP_CIMG_PK(TK_BF16, "bf16", 16, 16, 64, 3, 2),
    TK_BP_CIMG(TK_F16, "f16", 16, 16, 64, 3, 2),
    TK_BP_CIMG(TK_BF16, "bf16", 16, 16, 64, 3, 2),
    TK_BP_CIMG(TK_F32_COEF, "f32c", 16, 16, 64, 2, 2),
    TK_BP_CIMG(TK_F16, "f16", 16, 16, 32, 3, 3),
    TK_BP_CIMG(TK_F16, "f16", 32, 8, 64, 3, 2),
    TK_BP_CIMG_PK(TK_F16, "f16", 16, 16, 48, 3, 2),
    TK_BP_CIMG(TK_F32_COEF, "f32c", 16, 16, 32, 3, 2),
    TK_BP_CIMG(TK_F32_COEF, "f32c", 16, 16, 32, 2, 3),
    // two-stage twins of the 16-bit general walks, taken where three staged boxes would leave
    // room for one CTA per SM only (two_stage_twin)
    TK_BP_CIMG_F(TK_F16, "f16", 16, 16, 64, 2, 2),
    TK_BP_CIMG_F(TK_BF16, "bf16", 16, 16, 64, 2, 2),
};

static int g_variant_override = -1;  // index into kVariants, set by tk_bp_select_variant
static int g_diag_box_shrink = 0;    // rows taken off every staged box (tk_diag_shrink_box)
static int g_fp_variant = 0;  // forward projector: 0 slice lanes, fixed-point box; 1 column lanes; 2 slice lanes,
                              // FP32 atomics

static const BPVariant *pick_variant(int precision)
{
    if (g_variant_override >= 0 && kVariants[g_variant_override].precision == precision)
        return &kVariants[g_variant_override];
    for (const auto &v : kVariants)
        if (v.precision == precision) return &v;
    return nullptr;
}

// The two-stage variant with v's walk, storage and tile shape (the same
// arithmetic, so the same bits), or null.
static const BPVariant *two_stage_twin(const BPVariant *v)
{
    const char *lt = std::strchr(v->name, '<');
    const size_t np = lt ? (size_t)(lt - v->name) : std::strlen(v->name);
    for (const auto &c : kVariants)
        if (&c != v && c.precision == v->precision && c.coef == v->coef && !c.qcap && c.STAGES == 2 &&
            c.TX == v->TX && c.TY == v->TY && c.TZ == v->TZ && std::strncmp(c.name, v->name, np) == 0 &&
            c.name[np] == '<')
            return &c;
    return nullptr;
}

// Analytic bound of a tile's footprint extent (see the derivation in the
// design notes): for two voxels of one tile,
//   |du| <= s*dxy*Umax + Rmax*D/(D-Rmax)^2*s*dxy,
//   |dv| <= s*(TZ-1)*Umax + |aZ|max*D/(D-Rmax)^2*s*dxy.
int bp_box_dims(const tk_geometry &g, int nz, float zoff, int TX, int TY, int TZ, bool coef, int align, int *BW,
                int *BH)
{
    const double s = std::fabs((double)g.scale), D = g.D;
    const double ex = s * std::fmax(std::fabs(0.0 - g.cx), std::fabs((double)(g.X - 1) - g.cx)) + 1.0;
    const double ey = s * std::fmax(std::fabs(0.0 - g.cy), std::fabs((double)(g.Y - 1) - g.cy)) + 1.0;
    const double R = std::sqrt(ex * ex + ey * ey);
    TK_CHECK(D - R > 1e-3 * D, TK_ERR_UNSUPPORTED,
             "volume corners (radius %.1f px) reach the source (D = %.1f px)", R, D);
    const double Umax = D / (D - R), dU = D / ((D - R) * (D - R));
    const double dxy = s * std::sqrt((double)(TX - 1) * (TX - 1) + (double)(TY - 1) * (TY - 1));
    const double azmax = s * std::fmax(std::fabs((double)zoff), std::fabs((double)(nz - 1) + zoff)) + 1.0;
    const double du = dxy * Umax + R * dU * dxy;
    const double dv = s * (TZ - 1) * Umax + azmax * dU * dxy;
    // Sample boxes need columns floor(umin)-1 .. floor(umax)+1 plus the rounding
    // of the origin to the TMA granularity; coefficient entries cover a cell,
    // so their box is one column and one row smaller.  One extra of each
    // absorbs FP32-vs-FP64 differences of the device's corner evaluation.
    int bw = (int)std::floor(du) + (coef ? 4 : 5) + align;
    bw = (bw + align - 1) / align * align;
    int bh = (int)std::floor(dv) + (coef ? 5 : 7);
    TK_CHECK(bw <= 256 && bh <= 256, TK_ERR_UNSUPPORTED,
             "tile footprint %dx%d exceeds the 256x256 TMA box", bw, bh);
    *BW = bw;
    *BH = bh;
    return TK_OK;
}

// The quarter-turn kernel's conditions: a square volume of whole 32-column
// tile pairs centred on the axis (cx = cy = (X-1)/2 exactly, so a turn maps
// voxel coordinates onto each other exactly), no x/y flip, all angles in one
// launch with projection (q + k N/4) mod N at beta_q + k pi/2 (mod 2 pi) to within 1e-5 rad
// (angles as build_trig forms them; 1e-5 rad is 0.01 pixel at 1000 pixels
// from the axis), and a box that fits its slot.
static bool quad_eligible(const tk_geometry &g, int nz, float zoff, int angle0, int cap, int TY, int TZ,
                          int precision)
{
    if (g.X != g.Y || g.X % 32 != 0 || g.dirx || g.diry) return false;
    if (g.W >= (1 << 14) || g.H >= (1 << 14)) return false;  // footprint origins kept as 16-bit pairs
    if (g.cx != g.cy || g.cx != (float)(0.5 * (g.X - 1))) return false;
    if (g.N % 4 != 0 || g.N > kMaxParamProj) return false;
    const int nq = g.N / 4;
    auto beta = [&](int b) { return (double)(float)((float)(angle0 + b) * g.dfi + g.rot); };
    for (int q = 0; q < g.N; ++q)
        for (int k = 1; k < 4; ++k) {
            const double d = std::remainder(beta((q + k * nq) % g.N) - beta(q) - k * (M_PI / 2), 2 * M_PI);
            if (std::fabs(d) > 1e-5) return false;
        }
    const int ES = (int)entry_size(precision);
    int BW = 0, BH = 0;
    if (bp_box_dims(g, nz, zoff, 16, TY, TZ, true, 16 / ES, &BW, &BH) != TK_OK) return false;
    return BW * BH * ES <= cap;
}

// The quarter-turn variant for this launch: the selected variant if it is one
// (and fits), else, with no selection, the first automatic one whose box
// capacity holds the tile footprint; nullptr when none applies.
static const BPVariant *pick_quad(const tk_geometry &g, int precision, int nz, float zoff, int angle0)
{
    if (g_variant_override >= 0 && kVariants[g_variant_override].precision == precision) {
        const BPVariant *v = &kVariants[g_variant_override];
        return v->qcap && quad_eligible(g, nz, zoff, angle0, v->qcap, v->TY, v->TZ, precision) ? v : nullptr;
    }
    for (const auto &c : kVariants)
        if (c.precision == precision && c.qcap && c.qauto &&
            quad_eligible(g, nz, zoff, angle0, c.qcap, c.TY, c.TZ, precision))
            return &c;
    return nullptr;
}

// qlen < 0: the variant the precision picks (the quarter-turn kernel over all
// angles when the geometry allows it); qlen > 0: the quarter-turn kernel over
// the quarter-turn images of angles [qbase, qbase + qlen) only.
static int launch_bp_impl(const tk_geometry &g, const void *d_q, int precision, const float *d_q_scale, int nz,
                          float zoff, float *d_vol, int accumulate, cudaStream_t stream, int angle0, int qbase,
                          int qlen, bool compact = false)
{
    if (int rc = validate_geometry(&g)) return rc;
    TK_CHECK(d_q && d_vol, TK_ERR_INVALID, "backproject: null device pointer");
    TK_CHECK(nz >= 0, TK_ERR_INVALID, "backproject: nz < 0");
    TK_CHECK(valid_precision(precision), TK_ERR_INVALID, "backproject: unknown precision %d", precision);
    TK_CHECK((precision != TK_F16 && precision != TK_BF16) || d_q_scale, TK_ERR_INVALID,
             "backproject: 16-bit storage needs its scale");
    if (nz == 0) return TK_OK;
    const BPVariant *v = pick_variant(precision);
    TK_CHECK(v, TK_ERR_INVALID, "backproject: unknown precision %d", precision);
    if (qlen > 0) {  // the quarter-turn kernel on a quarter-turn-closed subset
        v = pick_quad(g, precision, nz, zoff, angle0);
        TK_CHECK(v, TK_ERR_UNSUPPORTED, "backproject: no quarter-turn symmetry for this geometry");
        TK_CHECK(qbase >= 0 && qbase + qlen <= g.N / 4, TK_ERR_INVALID, "backproject: angle range outside a quarter");
    } else if (v->qcap) {  // a quarter-turn variant that applies, else the format's general walk
        const BPVariant *w = pick_quad(g, precision, nz, zoff, angle0);
        if (!w)
            for (const auto &c : kVariants)
                if (c.precision == precision && !c.qcap) {
                    w = &c;
                    break;
                }
        v = w;
        TK_CHECK(v, TK_ERR_INVALID, "backproject: no general variant for precision %d", precision);
    }
    const bool quad = v->qcap > 0;
    auto encode = get_encode_fn();
    TK_CHECK(encode, TK_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");

    // TMA x-coordinate granularity in entries: 16 bytes
    const int ES = (int)entry_size(precision);
    const int align = v->coef ? (ES >= 16 ? 1 : 16 / ES) : 4;
    int BW, BH;
    if (int rc = bp_box_dims(g, nz, zoff, v->TX, v->TY, v->TZ, v->coef, align, &BW, &BH)) return rc;
    // A 16-bit general walk whose three staged boxes would fit one CTA per SM only (large
    // footprints: scale near 1.5 at high magnification) takes its two-stage twin, which keeps two.
    if (v->coef && !quad && v->STAGES == 3 && g_variant_override < 0 && precision != TK_F32_COEF) {
        int dev = 0, per_sm = 0;
        TK_CUDA(cudaGetDevice(&dev));
        TK_CUDA(cudaDeviceGetAttribute(&per_sm, cudaDevAttrMaxSharedMemoryPerMultiprocessor, dev));
        const size_t box = (size_t)((BW * BH + 15) / 16 * 16) * ES;
        const size_t fixed = (size_t)std::min(g.N, kMaxParamProj) * sizeof(int2) + 3 * sizeof(uint64_t) + 16;
        if (3 * box + fixed + 1024 > (size_t)per_sm / 2)  // 1 KB reserved per CTA
            if (const BPVariant *t = two_stage_twin(v)) v = t;
    }
    BH = std::max(1, BH - g_diag_box_shrink);  // 0 unless a self-check test shrinks the staged box
    TK_CHECK(!v->coef || BW * ES / 4 <= 256, TK_ERR_UNSUPPORTED, "tile footprint of %d entries too wide", BW);

    TK_CHECK(angle0 >= 0, TK_ERR_INVALID, "backproject: negative first angle index");
    std::vector<float> cs(g.N), sn(g.N);
    build_trig(g, cs.data(), sn.data(), angle0);
    const int p = reference_pad_length(g.W);

    const int tilesX = (g.X + v->TX - 1) / v->TX, tilesY = (g.Y + v->TY - 1) / v->TY;
    const int zchunks = (nz + v->TZ - 1) / v->TZ;
    TK_CHECK((long long)tilesX * tilesY < (1ll << 31) && zchunks < 65536, TK_ERR_UNSUPPORTED,
             "volume too large for one launch");

    const int pitch = storage_pitch(g.W, precision);
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
    P.stage_elems = v->coef ? (BW * BH + 15) / 16 * 16   // 128-byte aligned stages
                            : (BW * BH + 63) / 64 * 64;
    P.tilesX = tilesX;
    P.tilesY = tilesY;
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
    P.halfW = (float)g.W * 0.5f;
    // result *= delta_f * scaling, with scaling = 1/p (kernel.cu:113, 575)
    P.fscale = g.dfi * (1.f / (float)p);
    P.q_scale = (precision == TK_F16 || precision == TK_BF16) ? d_q_scale : nullptr;
    P.qbase = qlen > 0 ? qbase : 0;
    P.qlen = qlen > 0 ? qlen : g.N / 4;
    P.qf0 = compact ? 0 : P.qbase;
    P.qfs = compact ? P.qlen : g.N / 4;
    TK_CHECK(!compact || (quad && qlen > 0), TK_ERR_INVALID, "backproject: a compact image needs the quarter-turn kernel");

    const bool partial = v->coef && nz < v->TZ;
    const void *fn = partial ? v->fn_partial : v->fn;
    for (int b0 = 0; b0 < g.N; b0 += kMaxParamProj) {
        const int nb = std::min(kMaxParamProj, g.N - b0);
        P.N = nb;
        for (int b = 0; b < nb; ++b) P.trig[b] = make_float2(cs[b0 + b], sn[b0 + b]);
        P.accumulate = (accumulate || b0 > 0) ? 1 : 0;

        // Samples are FP32 elements; coefficient entries are viewed as ES/4 floats.
        const int fpe = v->coef ? ES / 4 : 1;
        CUtensorMap tmap;
        const char *base = static_cast<const char *>(d_q) + (size_t)b0 * g.H * pitch * ES;
        // (a compact quarter-turn image holds the four ranges' 4 qlen frames only)
        cuuint64_t dims[3] = {(cuuint64_t)g.W * fpe, (cuuint64_t)g.H, (cuuint64_t)(compact ? 4 * P.qlen : nb)};
        cuuint64_t strides[2] = {(cuuint64_t)pitch * ES, (cuuint64_t)pitch * g.H * ES};
        cuuint32_t box[3] = {(cuuint32_t)(BW * fpe), (cuuint32_t)BH, 1};
        cuuint32_t estr[3] = {1, 1, 1};
        CUresult cr = encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, const_cast<char *>(base), dims, strides, box,
                             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        TK_CHECK(cr == CUDA_SUCCESS, TK_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)cr);

        size_t smem = quad ? (size_t)v->STAGES * 4 * v->qcap : (size_t)v->STAGES * P.stage_elems * ES;
        // (the quarter-turn kernel keeps 4 qlen <= nb footprint origins as 16-bit pairs)
        smem += (size_t)nb * (quad ? sizeof(short2) : sizeof(int2)) + (size_t)v->STAGES * sizeof(uint64_t) + 16;
        TK_CHECK(smem <= 227 * 1024, TK_ERR_UNSUPPORTED, "backproject: %zu B of shared memory needed", smem);
        TK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        // the quarter-turn kernel: one CTA per orbit of four tiles (a first-quadrant tile)
        const unsigned ntiles = quad ? (unsigned)((tilesX / 2) * (tilesY / 2)) : (unsigned)(tilesX * tilesY);
        dim3 grid(ntiles, partial ? 1u : (unsigned)zchunks, 1);
        dim3 block((unsigned)(v->TX * v->TY), 1, 1);
        void *args[] = {&tmap, &P};
        TK_CUDA(cudaLaunchKernel(fn, grid, block, args, smem, stream));
        count_launch();
    }
    return TK_OK;
}

int launch_backproject(const tk_geometry &g, const void *d_q, int precision, const float *d_q_scale, int nz,
                       float zoff, float *d_vol, int accumulate, cudaStream_t stream, int angle0)
{
    return launch_bp_impl(g, d_q, precision, d_q_scale, nz, zoff, d_vol, accumulate, stream, angle0, 0, -1);
}

bool backproject_quarter_ok(const tk_geometry &g, int precision, int nz, float zoff)
{
    if (precision == TK_F32 || nz <= 0) return false;
    const BPVariant *v = pick_variant(precision);  // honours a selected variant
    return v && v->qcap && pick_quad(g, precision, nz, zoff, 0) != nullptr;
}

int launch_backproject_quarter(const tk_geometry &g, const void *d_q, int precision, const float *d_q_scale, int nz,
                               float zoff, float *d_vol, int accumulate, cudaStream_t stream, int qbase, int qlen,
                               bool compact)
{
    TK_CHECK(qlen > 0, TK_ERR_INVALID, "backproject: empty angle range");
    return launch_bp_impl(g, d_q, precision, d_q_scale, nz, zoff, d_vol, accumulate, stream, 0, qbase, qlen,
                          compact);
}

int launch_forward_project(const tk_geometry &g, const float *d_vol, int nz, float zoff, float *d_qbar,
                           int accumulate, cudaStream_t stream)
{
    constexpr int TX = 16, TY = 16, TZ = 32;
    if (int rc = validate_geometry(&g)) return rc;
    TK_CHECK(d_vol && d_qbar, TK_ERR_INVALID, "forward project: null device pointer");
    TK_CHECK(nz >= 0, TK_ERR_INVALID, "forward project: nz < 0");
    auto encode = get_encode_fn();
    TK_CHECK(encode, TK_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    const int Wp = row_pitch(g.W);
    if (!accumulate)
        TK_CUDA(cudaMemsetAsync(d_qbar, 0, (size_t)g.N * g.H * Wp * sizeof(float), stream));
    if (nz == 0) return TK_OK;

    const BPVariant shape = {nullptr, nullptr, TK_F32, TX, TY, TZ, 2, false, "fp"};
    int BW, BH;
    if (int rc = bp_box_dims(g, nz, zoff, shape.TX, shape.TY, shape.TZ, shape.coef, 4, &BW, &BH)) return rc;
    std::vector<float> cs(g.N), sn(g.N);
    build_trig(g, cs.data(), sn.data());
    const int p = reference_pad_length(g.W);
    const int tilesX = (g.X + TX - 1) / TX, tilesY = (g.Y + TY - 1) / TY;
    const int zchunks = (nz + TZ - 1) / TZ;
    TK_CHECK((long long)tilesX * tilesY < (1ll << 31) && zchunks < 65536, TK_ERR_UNSUPPORTED,
             "volume too large for one launch");
    const bool partial = nz < TZ;
    // Slice lanes with the two-word fixed-point box (variant 0, the default), column lanes (1), or
    // slice lanes with FP32 shared atomics (2).  The fixed-point box needs a bound on the contributions that
    // reach one cell of one projection from one tile (a cell takes the voxels whose u lies in a
    // 2-pixel band and whose v lies in a 2-row band):
    //  - the columns whose u falls in a 2-pixel band lie between two rays from the source, a strip
    //    at most w = 2 / (U_min |scale|) voxels wide; a 16 x 16 grid holds at most
    //    16 (floor(sqrt(2) w) + 1) points of such a strip (per grid line, floor(w / max(|cos|,
    //    |sin|)) + 1 points), and at most 256;
    //  - per column, the slices whose row falls in a 2-row band, at most floor(2 / dv_min) + 2,
    //    dv_min = |scale| U_min the smallest row step, and at most the 32 slices of a chunk;
    //  with U = D / (D - S), |S| < W/2 inside the FOV: U_min = D / (D + W/2), U_max = D / (D - W/2).
    const bool cols = g_fp_variant != 1;
    const double hw = 0.5 * g.W;
    const bool fixed = g_fp_variant == 0 && (double)g.D > hw;  // else U has no bound: FP32 atomics
    int cbits = 0;
    float u2max = 0.f;
    if (fixed) {
        const double umin = g.D / (g.D + hw), umax = g.D / (g.D - hw);
        const double dv_min = std::max(std::fabs((double)g.scale) * umin, 1e-6);
        const double ncols = std::min(256.0, 16.0 * (std::floor(std::sqrt(2.0) * 2.0 / dv_min) + 1.0));
        const double count = ncols * std::min(32.0, std::floor(2.0 / dv_min) + 2.0);
        while ((double)(1 << cbits) < count) ++cbits;  // <= 13
        u2max = (float)(1.0001 * umax * umax);
    }
    const void *fn;
    if (!cols)
        fn = partial ? reinterpret_cast<const void *>(&fp_scatter_kernel<TX, TY, true>)
                     : reinterpret_cast<const void *>(&fp_scatter_kernel<TX, TY, false>);
    else if (fixed && cbits <= 8)
        fn = partial ? reinterpret_cast<const void *>(&fp_scatter_col_kernel<TX, TY, true, 3>)
                     : reinterpret_cast<const void *>(&fp_scatter_col_kernel<TX, TY, false, 3>);
    else if (fixed && cbits <= 9)
        fn = partial ? reinterpret_cast<const void *>(&fp_scatter_col_kernel<TX, TY, true, 2>)
                     : reinterpret_cast<const void *>(&fp_scatter_col_kernel<TX, TY, false, 2>);
    else if (fixed)
        fn = partial ? reinterpret_cast<const void *>(&fp_scatter_col_kernel<TX, TY, true, 1>)
                     : reinterpret_cast<const void *>(&fp_scatter_col_kernel<TX, TY, false, 1>);
    else
        fn = partial ? reinterpret_cast<const void *>(&fp_scatter_col_kernel<TX, TY, true, 0>)
                     : reinterpret_cast<const void *>(&fp_scatter_col_kernel<TX, TY, false, 0>);

    static thread_local BPParams P;
    std::memset(&P, 0, sizeof(P));
    P.err = device_error_word();
    TK_CHECK(P.err, TK_ERR_CUDA, "device error word unavailable");
    P.slice_stride = (long long)g.X * g.Y;
    P.X = g.X;
    P.Y = g.Y;
    P.nz = nz;
    P.BW = BW;
    P.BH = BH;
    P.stage_elems = (BW * BH + 31) / 32 * 32;  // 128-byte aligned boxes
    P.tilesX = tilesX;
    P.tilesY = tilesY;
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
    P.halfW = (float)g.W * 0.5f;
    P.fscale = g.dfi * (1.f / (float)p);  // the backprojection's scale, transposed

    for (int b0 = 0; b0 < g.N; b0 += kMaxParamProj) {
        const int nb = std::min(kMaxParamProj, g.N - b0);
        P.N = nb;
        for (int b = 0; b < nb; ++b) P.trig[b] = make_float2(cs[b0 + b], sn[b0 + b]);
        CUtensorMap tmap;
        char *base = reinterpret_cast<char *>(d_qbar) + (size_t)b0 * g.H * Wp * sizeof(float);
        cuuint64_t dims[3] = {(cuuint64_t)g.W, (cuuint64_t)g.H, (cuuint64_t)nb};
        cuuint64_t strides[2] = {(cuuint64_t)Wp * 4, (cuuint64_t)Wp * g.H * 4};
        cuuint32_t box[3] = {(cuuint32_t)BW, (cuuint32_t)BH, 1};
        cuuint32_t estr[3] = {1, 1, 1};
        CUresult cr = encode(&tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, base, dims, strides, box, estr,
                             CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        TK_CHECK(cr == CUDA_SUCCESS, TK_ERR_CUDA, "cuTensorMapEncodeTiled failed (%d)", (int)cr);
        // odd-pitch accumulation box (two words per cell in the fixed-point form)
        const size_t acc_elems = (size_t)((BH * (BW + 1) + 31) & ~31) * (fixed ? 2 : 1);
        const size_t geo_bytes = cols ? (size_t)(TX * TY / 32) * 32 * sizeof(float4) : 0;  // slice-lane form
        const size_t smem = (2 * (size_t)P.stage_elems + acc_elems) * sizeof(float) + geo_bytes +
                            (size_t)nb * sizeof(int2) + 16;
        TK_CHECK(smem <= 227 * 1024, TK_ERR_UNSUPPORTED, "forward project: %zu B of shared memory needed", smem);
        TK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
        dim3 grid((unsigned)(tilesX * tilesY), partial ? 1u : (unsigned)zchunks, 1);
        const float *vin = d_vol;
        float u2 = u2max;
        int cb = cbits;
        void *args_cols[] = {&tmap, &P, &vin, &u2, &cb};
        void *args_rows[] = {&tmap, &P, &vin};
        TK_CUDA(cudaLaunchKernel(fn, grid, dim3(TX * TY), cols ? args_cols : args_rows, smem, stream));
        count_launch();
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

extern "C" int tk_fp_select_variant(int i)
{
    if (i < 0 || i > 2) {
        tk::set_error("no forward-projector variant %d", i);
        return TK_ERR_INVALID;
    }
    tk::g_fp_variant = i;
    return TK_OK;
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

extern "C" int tk_diag_shrink_box(int rows)
{
    if (rows < 0) {
        tk::set_error("tk_diag_shrink_box: rows < 0");
        return TK_ERR_INVALID;
    }
    tk::g_diag_box_shrink = rows;
    return TK_OK;
}
