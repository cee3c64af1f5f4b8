// tk_bp_core.cuh -- device pieces shared by the backprojection kernels
// (per-volume kernels in tk_bp.cu, the batched persistent kernel in
// tk_batch.cu): axis sign flips, the coefficient-image storage traits and
// the z-column update.
#pragma once

#include "tk_common.cuh"

namespace tk {

__device__ __forceinline__ float flip(float v, unsigned mask)
{
    return __uint_as_float(__float_as_uint(v) ^ mask);
}

// Tile of CTA index i: tiles are visited in column groups kTileGroup tiles
// wide (row by row inside a group), so the CTAs resident at one time cover a
// compact patch of the slice whose footprints overlap in L2, rather than a
// thin strip across the whole slice.
constexpr int kTileGroup = 16;
__device__ __forceinline__ int2 tile_of(int i, int tilesX, int tilesY)
{
    const int per = kTileGroup * tilesY;
    const int g = i / per, r = i - g * per;
    const int w = min(kTileGroup, tilesX - g * kTileGroup);  // the last group may be narrower
    return make_int2(g * kTileGroup + r % w, r / w);
}

// Per column-angle geometry with every rounding spelled out:
//   S = aX cos + aY sin,  T = aY cos - aX sin,  U = D / (D - S),  u = T U + cX
// (kernel.cu:102-109).  Every kernel evaluates it through this function --
// the per-volume backprojectors, the batched kernel and the forward
// projector that must be their exact transpose -- so they get the same bits
// whatever FMA contraction the compiler would otherwise pick per kernel.
__device__ __forceinline__ void column_geometry(float aX, float aY, float2 cs, float D, float cX, float &U, float &u)
{
    const float S = fmaf(aX, cs.x, __fmul_rn(aY, cs.y));
    const float T = fmaf(aY, cs.x, -__fmul_rn(aX, cs.y));
    U = __fdiv_rn(D, __fsub_rn(D, S));
    u = fmaf(T, U, cX);
}
// Detector row of slice coordinate aZ: aZ U + cZ with one rounding.
__device__ __forceinline__ float slice_v(float aZ, float U, float cZ) { return fmaf(aZ, U, cZ); }

// Coefficient-image storage (see tk_precision): entry (r, c) covers the
// detector cell [r, r+1] x [c, c+1], so an update is one shared load of one
// entry and
//   A = Q + fu dU,  B = dV + fu dUV,  acc += U^2 (A + fv B)
// (16-bit storage: the four values converted to FP32 first, eval_f32; the
// selectable half-math forms take A and B from one packed HFMA2, eval).
// Loads use 32-bit shared
// addresses (inline PTX) so the address of an update is one IMAD.
template <int PREC> struct Cimg;
template <> struct Cimg<TK_F32_COEF> {
    static constexpr int kBytes = 16, kAlign = 1;
    static __device__ __forceinline__ float2 eval(uint32_t addr, float fu, float2)
    {
        float q, du, dv, duv;
        asm volatile("ld.shared.v4.f32 {%0, %1, %2, %3}, [%4];" : "=f"(q), "=f"(du), "=f"(dv), "=f"(duv) : "r"(addr));
        return make_float2(fmaf(fu, du, q), fmaf(fu, duv, dv));
    }
    static __device__ __forceinline__ float2 eval_f32(uint32_t addr, float fu) { return eval(addr, fu, float2{}); }
};
// The two halves of a 16-bit pair word as FP32 (exact conversions): lo is
// the half in bits 0-15.
template <int PREC> __device__ __forceinline__ void unpack_pair(uint32_t w, float &lo, float &hi)
{
    if constexpr (PREC == TK_BF16) {
        // a bfloat16 is the upper half of its FP32 value: two byte permutes (integer pipe)
        uint32_t l, h;
        asm("prmt.b32 %0, %2, 0, 0x1044;\n\t"
            "prmt.b32 %1, %2, 0, 0x3244;"
            : "=r"(l), "=r"(h)
            : "r"(w));
        lo = __uint_as_float(l);
        hi = __uint_as_float(h);
    } else {
        const float2 f = __half22float2(*reinterpret_cast<const __half2 *>(&w));
        lo = f.x;
        hi = f.y;
    }
}
// FP32 interpolation of a 16-bit entry {(Q, dV), (dU, dUV)}: the four values
// converted exactly to FP32, then A = fma(fu, dU, Q), B = fma(fu, dUV, dV) --
// the operations of the FP32 coefficient format on the stored values.
template <int PREC> __device__ __forceinline__ float2 eval16_f32(uint32_t addr, float fu)
{
    uint32_t lo, hi;
    asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(lo), "=r"(hi) : "r"(addr));
    float q, dv, du, duv;
    unpack_pair<PREC>(lo, q, dv);
    unpack_pair<PREC>(hi, du, duv);
    return make_float2(fmaf(fu, du, q), fmaf(fu, duv, dv));
}
template <> struct Cimg<TK_F16> {
    static constexpr int kBytes = 8, kAlign = 2;
    static __device__ __forceinline__ float2 eval(uint32_t addr, float, float2 fu2raw)
    {
        uint32_t lo, hi;
        asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(lo), "=r"(hi) : "r"(addr));
        const __half2 h = __hfma2(*reinterpret_cast<const __half2 *>(&hi),
                                  *reinterpret_cast<const __half2 *>(&fu2raw.x),
                                  *reinterpret_cast<const __half2 *>(&lo));
        return __half22float2(h);
    }
    static __device__ __forceinline__ float2 eval_f32(uint32_t addr, float fu) { return eval16_f32<TK_F16>(addr, fu); }
};
template <> struct Cimg<TK_BF16> {
    static constexpr int kBytes = 8, kAlign = 2;
    static __device__ __forceinline__ float2 eval(uint32_t addr, float, float2 fu2raw)
    {
        uint32_t lo, hi;
        asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];" : "=r"(lo), "=r"(hi) : "r"(addr));
        const __nv_bfloat162 h = __hfma2(*reinterpret_cast<const __nv_bfloat162 *>(&hi),
                                         *reinterpret_cast<const __nv_bfloat162 *>(&fu2raw.x),
                                         *reinterpret_cast<const __nv_bfloat162 *>(&lo));
        return __bfloat1622float2(h);
    }
    static __device__ __forceinline__ float2 eval_f32(uint32_t addr, float fu) { return eval16_f32<TK_BF16>(addr, fu); }
};

// fu packed for the 16-bit HFMA2 (carried in the bits of a float2.x).
template <int PREC> __device__ __forceinline__ float2 pack_fu(float fu)
{
    float2 r = make_float2(0.f, 0.f);
    if constexpr (PREC == TK_F16) {
        const __half2 h = __float2half2_rn(fu);
        r.x = *reinterpret_cast<const float *>(&h);
    } else if constexpr (PREC == TK_BF16) {
        const __nv_bfloat162 h = __float2bfloat162_rn(fu);
        r.x = *reinterpret_cast<const float *>(&h);
    }
    return r;
}

// One column's update over a TZ-voxel z walk, v_z = v0 + z dv, reading the
// entries of the staged box at sbase (shared address, already offset by the
// column and by -(kMagicBits + box row origin) rows).
// Floor and fraction of two row coordinates with packed FP32 (one
// add.rm.f32x2 and two sub.f32x2 for both lanes); per lane the same IEEE
// operations as the scalar walk: fl = RD(v + M), fv = v - (fl - M).
__device__ __forceinline__ void floor_frac_x2(float va, float vb, float &fla, float &flb, float &fva, float &fvb)
{
    asm("{\n\t.reg .b64 V, M, F, T;\n\t"
        "mov.b64 V, {%4, %5};\n\t"
        "mov.b64 M, {%6, %6};\n\t"
        "add.rm.f32x2 F, V, M;\n\t"
        "sub.rn.f32x2 T, F, M;\n\t"
        "sub.rn.f32x2 T, V, T;\n\t"
        "mov.b64 {%0, %1}, F;\n\t"
        "mov.b64 {%2, %3}, T;\n\t}"
        : "=f"(fla), "=f"(flb), "=f"(fva), "=f"(fvb)
        : "f"(va), "f"(vb), "f"(kMagic));
}
// (va, vb) += (d, d) as one add.rn.f32x2.
__device__ __forceinline__ void add_pair(float &va, float &vb, float d)
{
    asm("{\n\t.reg .b64 V, D;\n\t"
        "mov.b64 V, {%0, %1};\n\t"
        "mov.b64 D, {%2, %2};\n\t"
        "add.rn.f32x2 V, V, D;\n\t"
        "mov.b64 {%0, %1}, V;\n\t}"
        : "+f"(va), "+f"(vb)
        : "f"(d));
}
// acc_i = fma(w_i, fma(fv_i, b_i, a_i), acc_i) for i = 0, 1 as two fma.rn.f32x2.
__device__ __forceinline__ void interp_acc_x2(float aa, float ab, float ba, float bb, float fva, float fvb, float wa,
                                              float wb, float &acc0, float &acc1)
{
    asm("{\n\t.reg .b64 A, B, FV, W, C;\n\t"
        "mov.b64 A, {%2, %3};\n\t"
        "mov.b64 B, {%4, %5};\n\t"
        "mov.b64 FV, {%6, %7};\n\t"
        "mov.b64 W, {%8, %9};\n\t"
        "mov.b64 C, {%0, %1};\n\t"
        "fma.rn.f32x2 A, FV, B, A;\n\t"
        "fma.rn.f32x2 C, W, A, C;\n\t"
        "mov.b64 {%0, %1}, C;\n\t}"
        : "+f"(acc0), "+f"(acc1)
        : "f"(aa), "f"(ab), "f"(ba), "f"(bb), "f"(fva), "f"(fvb), "f"(wa), "f"(wb));
}

// FP32 bilinear interpolation and accumulation of two slices a, b from their
// entries' four values (Q, dU, dV, dUV) as four fma.rn.f32x2; per lane
//   A = fma(fu, dU, Q), B = fma(fu, dUV, dV), acc = fma(w, fma(fv, B, A), acc),
// the operations of Cimg<TK_F32_COEF>::eval followed by interp_acc_x2.
__device__ __forceinline__ void interp4_acc_x2(float qa, float qb, float dua, float dub, float dva, float dvb,
                                               float duva, float duvb, float fu, float fva, float fvb, float wa,
                                               float wb, float &acc0, float &acc1)
{
    asm("{\n\t.reg .b64 Q, DU, DV, DUV, FU, FV, W, C;\n\t"
        "mov.b64 Q, {%2, %3};\n\t"
        "mov.b64 DU, {%4, %5};\n\t"
        "mov.b64 DV, {%6, %7};\n\t"
        "mov.b64 DUV, {%8, %9};\n\t"
        "mov.b64 FU, {%10, %10};\n\t"
        "mov.b64 FV, {%11, %12};\n\t"
        "mov.b64 W, {%13, %14};\n\t"
        "mov.b64 C, {%0, %1};\n\t"
        "fma.rn.f32x2 Q, FU, DU, Q;\n\t"
        "fma.rn.f32x2 DV, FU, DUV, DV;\n\t"
        "fma.rn.f32x2 Q, FV, DV, Q;\n\t"
        "fma.rn.f32x2 C, W, Q, C;\n\t"
        "mov.b64 {%0, %1}, C;\n\t}"
        : "+f"(acc0), "+f"(acc1)
        : "f"(qa), "f"(qb), "f"(dua), "f"(dub), "f"(dva), "f"(dvb), "f"(duva), "f"(duvb), "f"(fu), "f"(fva),
          "f"(fvb), "f"(wa), "f"(wb));
}

// FP32 bilinear interpolation and accumulation of two slices a, b from their
// 16-bit entries {(Q, dV), (dU, dUV)} (low word, high word), the values
// converted exactly to FP32; per slice
//   A = fma(fu, dU, Q), B = fma(fu, dUV, dV), acc = fma(w, fma(fv, B, A), acc):
// the operations of interp4_acc_x2 as scalar FMAs (same bits).
template <int PREC>
__device__ __forceinline__ void interp_scalar_acc(uint32_t loa, uint32_t hia, uint32_t lob, uint32_t hib, float fu,
                                                  float fva, float fvb, float wa, float wb, float &acc0, float &acc1)
{
    float qa, dva, dua, duva, qb, dvb, dub, duvb;
    unpack_pair<PREC>(loa, qa, dva);
    unpack_pair<PREC>(hia, dua, duva);
    unpack_pair<PREC>(lob, qb, dvb);
    unpack_pair<PREC>(hib, dub, duvb);
    const float Aa = fmaf(fu, dua, qa), Ba = fmaf(fu, duva, dva);
    const float Ab = fmaf(fu, dub, qb), Bb = fmaf(fu, duvb, dvb);
    acc0 = fmaf(wa, fmaf(fva, Ba, Aa), acc0);
    acc1 = fmaf(wb, fmaf(fvb, Bb, Ab), acc1);
}

// acc0 += w.lo * val.lo and acc1 += w.hi * val.hi: FP16 products (exact in
// FP32) added to FP32 accumulators with one rounding (fma.rn.f32.f16).
__device__ __forceinline__ void acc_mixed_x2(uint32_t val2, uint32_t w2, float &acc0, float &acc1)
{
    asm("{\n\t.reg .b16 vl, vh, wl, wh;\n\t"
        "mov.b32 {vl, vh}, %2;\n\t"
        "mov.b32 {wl, wh}, %3;\n\t"
        "fma.rn.f32.f16 %0, wl, vl, %0;\n\t"
        "fma.rn.f32.f16 %1, wh, vh, %1;\n\t}"
        : "+f"(acc0), "+f"(acc1)
        : "r"(val2), "r"(w2));
}

// The row interpolation and accumulation of two slices from their
// column-interpolated entries ha = (value, row derivative) of slice a and hb of
// slice b: acc0 += w.lo * (ha.lo + fv.lo * ha.hi), acc1 += w.hi * (hb.lo +
// fv.hi * hb.hi), each interpolation one FP16 FMA on half-selected operands (the
// same roundings as one HFMA2 on the regrouped halves, without regrouping them).
__device__ __forceinline__ void row_acc_x2(uint32_t ha, uint32_t hb, uint32_t fv2, uint32_t w2, float &acc0,
                                           float &acc1)
{
    asm("{\n\t.reg .b16 al, ah, bl, bh, fa, fb, wa, wb, va, vb;\n\t"
        "mov.b32 {al, ah}, %2;\n\t"
        "mov.b32 {bl, bh}, %3;\n\t"
        "mov.b32 {fa, fb}, %4;\n\t"
        "mov.b32 {wa, wb}, %5;\n\t"
        "fma.rn.f16 va, fa, ah, al;\n\t"
        "fma.rn.f16 vb, fb, bh, bl;\n\t"
        "fma.rn.f32.f16 %0, wa, va, %0;\n\t"
        "fma.rn.f32.f16 %1, wb, vb, %1;\n\t}"
        : "+f"(acc0), "+f"(acc1)
        : "r"(ha), "r"(hb), "r"(fv2), "r"(w2));
}

// Walks of a column (WALK):
//   0  scalar FP32, one slice per step;
//   1  packed FP32, two slices per step (floor/frac, the row interpolation and
//      the accumulation as f32x2); per voxel exactly the operations of the
//      scalar walk, so both give the same bits;
//   2  FP16 storage only, two slices per step: the pair's row coordinates
//      advanced by (2 dv, 2 dv) with one add.f32x2 and set exactly,
//      fmaf(z, dv, v0), every 16 pairs (drift below 16 half-ulps of v between
//      them); floor/frac in FP32 as above;
//      the column interpolation of both entries by HFMA2, then the row
//      interpolation of both slices by one HFMA2 on the regrouped halves
//      (two permutes) with the fractions rounded to FP16, and the weight U^2
//      rounded to FP16 applied by fma.rn.f32.f16 into the FP32 accumulators.
//      Fewer FP32-pipe operations, FP16 rounding of fv, U^2 and the
//      interpolated sample;
//   3  walk 2 with each slice's row interpolation one FP16 FMA on
//      half-selected operands (row_acc_x2) instead of the permutes and the
//      HFMA2: the same roundings, so the same bits, and 4.5 % faster on the
//      1024^2 x 64-slice slab (the FP16 half-math walk, selectable);
//   4  16-bit storage with FP32 interpolation (the TK_F16 and TK_BF16
//      default): walk 1 with each entry's four values converted exactly to
//      FP32 and interpolated by interp4_acc_x2, so per voxel the operations of
//      the FP32 coefficient format on the stored values; PARTIAL chunks take
//      the scalar form of the same operations (Cimg::eval_f32).
template <int PREC, int TZ, bool ALL_IN, bool PARTIAL, int WALK = 0>
__device__ __forceinline__ void update_cimg(uint32_t sbase, uint32_t row_bytes, float v0, float dv, float fu,
                                            float U2, float Hm1, int zlast, float (&acc)[TZ])
{
    const float2 fu2 = pack_fu<PREC>(fu);
    if constexpr ((WALK == 2 || WALK == 3) && PREC == TK_F16 && !PARTIAL && (TZ % 2 == 0)) {
        const __half2 fuh = *reinterpret_cast<const __half2 *>(&fu2.x);
        const __half2 U2h2 = __float2half2_rn(U2);
        const uint32_t w_all = *reinterpret_cast<const uint32_t *>(&U2h2);
        const float dv2 = 2.f * dv;
        float ra = v0, rb = v0;
#pragma unroll
        for (int z = 0; z < TZ; z += 2) {
            float va, vb;
            if (z % 32 == 0) {
                va = fmaf((float)z, dv, v0);
                vb = fmaf((float)(z + 1), dv, v0);
            } else {
                add_pair(ra, rb, dv2);
                va = ra;
                vb = rb;
            }
            ra = va;
            rb = vb;
            float fla, flb, fva, fvb;
            floor_frac_x2(va, vb, fla, flb, fva, fvb);
            uint32_t loa, hia, lob, hib;
            asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];"
                         : "=r"(loa), "=r"(hia)
                         : "r"((uint32_t)__float_as_int(fla) * row_bytes + sbase));
            asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];"
                         : "=r"(lob), "=r"(hib)
                         : "r"((uint32_t)__float_as_int(flb) * row_bytes + sbase));
            // (A, B) = (Q, dV) + fu (dU, dUV) per slice, then (A_a, A_b) + fv (B_a, B_b)
            const __half2 ha = __hfma2(*reinterpret_cast<const __half2 *>(&hia), fuh,
                                       *reinterpret_cast<const __half2 *>(&loa));
            const __half2 hb = __hfma2(*reinterpret_cast<const __half2 *>(&hib), fuh,
                                       *reinterpret_cast<const __half2 *>(&lob));
            const __half2 fv2 = __floats2half2_rn(fva, fvb);
            uint32_t w2 = w_all;
            if constexpr (!ALL_IN) {  // kernel.cu:130-131
                w2 = ((va >= 0.f && va <= Hm1) ? (w_all & 0xffffu) : 0u) |
                     ((vb >= 0.f && vb <= Hm1) ? (w_all & 0xffff0000u) : 0u);
            }
            if constexpr (WALK == 2) {
                const __half2 val = __hfma2(fv2, __highs2half2(ha, hb), __lows2half2(ha, hb));
                acc_mixed_x2(*reinterpret_cast<const uint32_t *>(&val), w2, acc[z], acc[z + 1]);
            } else {  // the same roundings on half-selected operands (row_acc_x2)
                row_acc_x2(*reinterpret_cast<const uint32_t *>(&ha), *reinterpret_cast<const uint32_t *>(&hb),
                           *reinterpret_cast<const uint32_t *>(&fv2), w2, acc[z], acc[z + 1]);
            }
        }
    } else if constexpr (WALK == 4 && PREC != TK_F32_COEF && !PARTIAL && (TZ % 2 == 0)) {
#pragma unroll
        for (int z = 0; z < TZ; z += 2) {
            const float va = fmaf((float)z, dv, v0), vb = fmaf((float)(z + 1), dv, v0);
            float fla, flb, fva, fvb;
            floor_frac_x2(va, vb, fla, flb, fva, fvb);
            uint32_t loa, hia, lob, hib;
            asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];"
                         : "=r"(loa), "=r"(hia)
                         : "r"((uint32_t)__float_as_int(fla) * row_bytes + sbase));
            asm volatile("ld.shared.v2.u32 {%0, %1}, [%2];"
                         : "=r"(lob), "=r"(hib)
                         : "r"((uint32_t)__float_as_int(flb) * row_bytes + sbase));
            float qa, dva, dua, duva, qb, dvb, dub, duvb;
            unpack_pair<PREC>(loa, qa, dva);
            unpack_pair<PREC>(hia, dua, duva);
            unpack_pair<PREC>(lob, qb, dvb);
            unpack_pair<PREC>(hib, dub, duvb);
            float wa = U2, wb = U2;
            if constexpr (!ALL_IN) {
                wa = (va >= 0.f && va <= Hm1) ? U2 : 0.f;  // kernel.cu:130-131
                wb = (vb >= 0.f && vb <= Hm1) ? U2 : 0.f;
            }
            interp4_acc_x2(qa, qb, dua, dub, dva, dvb, duva, duvb, fu, fva, fvb, wa, wb, acc[z], acc[z + 1]);
        }
    } else if constexpr (WALK >= 1 && !PARTIAL && (TZ % 2 == 0)) {
#pragma unroll
        for (int z = 0; z < TZ; z += 2) {
            const float va = fmaf((float)z, dv, v0), vb = fmaf((float)(z + 1), dv, v0);
            float fla, flb, fva, fvb;
            floor_frac_x2(va, vb, fla, flb, fva, fvb);
            const float2 x = Cimg<PREC>::eval((uint32_t)__float_as_int(fla) * row_bytes + sbase, fu, fu2);
            const float2 y = Cimg<PREC>::eval((uint32_t)__float_as_int(flb) * row_bytes + sbase, fu, fu2);
            float wa = U2, wb = U2;
            if constexpr (!ALL_IN) {
                wa = (va >= 0.f && va <= Hm1) ? U2 : 0.f;  // kernel.cu:130-131
                wb = (vb >= 0.f && vb <= Hm1) ? U2 : 0.f;
            }
            interp_acc_x2(x.x, y.x, x.y, y.y, fva, fvb, wa, wb, acc[z], acc[z + 1]);
        }
    } else {
#pragma unroll
        for (int z = 0; z < TZ; ++z) {
            if (PARTIAL && z > zlast) break;
            const float v = fmaf((float)z, dv, v0);
            const float fl = __fadd_rd(v, kMagic);
            const float fv = v - (fl - kMagic);
            const uint32_t addr = (uint32_t)__float_as_int(fl) * row_bytes + sbase;
            const float2 ab = WALK == 4 ? Cimg<PREC>::eval_f32(addr, fu) : Cimg<PREC>::eval(addr, fu, fu2);
            const float val = fmaf(fv, ab.y, ab.x);
            if constexpr (ALL_IN) {
                acc[z] = fmaf(U2, val, acc[z]);
            } else {
                const float w = (v >= 0.f && v <= Hm1) ? U2 : 0.f;  // kernel.cu:130-131
                acc[z] = fmaf(w, val, acc[z]);
            }
        }
    }
}

}  // namespace tk
