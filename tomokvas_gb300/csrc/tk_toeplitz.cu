// tk_toeplitz.cu -- the ramp filter as a Toeplitz product on the tcgen05
// tensor cores (sm_103a).
//
// The reference filters each detector row by zero padding to p = 2 nextpow2(W),
// R2C, multiplying by tau |R2C(h)| and C2R unnormalised (fConvolution,
// FBPG/kernel.cu:557-781).  The spectrum is real and even, so this is the
// linear convolution q[c] = sum_j g[j] K[c - j] with the even kernel
//   K[m] = Hf[0] + Hf[p/2] (-1)^m + 2 sum_{k=1}^{p/2-1} Hf[k] cos(2 pi k m / p),
// and, since |c - j| < W <= p/2, a W x W symmetric Toeplitz matrix.  Here the
// rows of a tile are filtered as one GEMM on the tensor cores:
//
//   D[c][row] = sum_kappa T[c][kappa] G[row][kappa],   kappa = Wk - 1 - j,
//
// with the input columns reversed (Wk = W rounded up to 64).  T[c][kappa] =
// K[c + kappa - (Wk - 1)] then depends on c + kappa only (a Hankel matrix),
// so in the no-swizzle K-major core-matrix layout (8 rows x 16 bytes per core
// matrix) core (a, b) equals core (a + b): T is stored as one run of
// 16 mt + Wk/8 distinct 128-byte cores and addressed with a leading and a
// stride byte offset of 128 each.  Split-BF16 compensated products give FP32
// accuracy: g = g_hi + g_lo and T = T_hi + T_lo, each part bfloat16, and
//   D = T_hi G_hi + T_hi G_lo + T_lo G_hi
// accumulated in FP32 in tensor memory (the dropped T_lo G_lo is below 2^-16
// of the product).
//
// CTA roles (one CTA per SM, persistent over row tiles of R detector rows,
// consecutive tiles overlapping by one row so that every coefficient entry's
// next row is in its own tile; two accumulators of mt x R columns in tensor
// memory, so that a tile's MMAs run while the epilogue drains the previous
// tile's):
//   warps 0-7    producers: read the raw rows (uint16 counts or FP32 line
//                integrals; with 16-byte aligned rows copied into a per-thread
//                two-stage shared buffer with cp.async one group of four rows
//                ahead), apply flat field + log and the cosine weight
//                (the FFT filter's load, tk_filter_core.cuh), split into
//                bfloat16 parts and write 64-column chunks of G into a ring of
//                shared-memory slots (mbarriers full/empty);
//   warp 16      tensor-memory allocation and, from one lane, the MMAs:
//                per chunk 4 K-steps x 3 products x mt column tiles of
//                tcgen05.mma.cta_group::1.kind::f16 (M = 128 output columns,
//                N = R rows, K = 16) into the tile's accumulator (tile parity);
//                tcgen05.commit releases the slot, and after the last chunk
//                signals that accumulator;
//   warps 8-15   epilogue, two sets of four (TMEM lane quarters 0-3) taking
//                alternate 32-row chunks, each set with its own staging
//                buffer and named barrier: tcgen05.ld the accumulator, stage
//                it in shared memory, write the storage format (FP32 samples
//                or the bilinear coefficient image, scaled by the storage
//                scale) with each warp storing consecutive columns of one row.
// Every wait is bounded; a timeout sets ERR_WAIT_TIMEOUT and every role
// leaves its loop; the MMAs issued are drained before the tensor memory is
// freed.
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

constexpr int kToepMaxW = 512;        // one pass: the accumulator of mt x R <= 512 columns
constexpr int kToepKmax = 528;        // |m| <= max(Wk - 1, 128 mt + 7)
constexpr int kToepProdWarps = 8;
constexpr int kToepEpiWarps = 8;  // two sets of four (one per TMEM lane quarter), alternate chunks
constexpr int kToepThreads = (kToepProdWarps + kToepEpiWarps + 1) * 32;  // producers, epilogue, MMA
constexpr int kToepPitch = 132;       // epilogue staging row pitch (floats): 129 used, 16-byte rows

struct ToepParams {
    LoadParams L;
    void *out;
    const float *q_scale;    // storage scale (16-bit formats) or null
    unsigned *err;
    long long nrows;         // N * H detector rows
    long long ntiles;        // row tiles: ceil(nrows / (R - 1))
    int precision, pitch;    // output format and row pitch (entries or samples)
    int fgrp, fstride;       // frames in groups (see launch_filter)
    int Wk, nk, mt, R;       // K extent (multiple of 64), K chunks, output-column tiles, rows per tile
    int slots;               // ring depth
    int ncores;              // Hankel cores: 16 mt + Wk / 8
    int kmax;
    uint32_t tmem_cols;
    uint32_t idesc;          // instruction descriptor (BF16 x BF16 -> F32, M = 128, N = R, K-major)
    uint32_t khl[kToepKmax + 1];  // K[m], m = 0..kmax: bfloat16 hi (bits 0-15), lo (bits 16-31)
};

__device__ __forceinline__ void mbar_arrive(uint64_t *bar)
{
    asm volatile("mbarrier.arrive.shared::cta.b64 _, [%0];" ::"r"(smem_u32(bar)) : "memory");
}

// UMMA shared-memory descriptor, no swizzle (K-major core matrices of 8 rows x
// 16 bytes): start address, leading (K) and stride (M/N) byte offsets,
// descriptor version 1 (bits 46-47).
__device__ __forceinline__ uint64_t umma_desc(uint32_t saddr, uint32_t lbo, uint32_t sbo)
{
    return (uint64_t)((saddr & 0x3FFFFu) >> 4) | ((uint64_t)(lbo >> 4) << 16) | ((uint64_t)(sbo >> 4) << 32) |
           (1ull << 46);
}

__device__ __forceinline__ void umma_bf16(uint32_t d_tmem, uint64_t adesc, uint64_t bdesc, uint32_t idesc,
                                          uint32_t accumulate)
{
    asm volatile(
        "{\n\t.reg .pred p;\n\t"
        "setp.ne.b32 p, %4, 0;\n\t"
        "tcgen05.mma.cta_group::1.kind::f16 [%0], %1, %2, %3, p;\n\t}" ::"r"(d_tmem),
        "l"(adesc), "l"(bdesc), "r"(idesc), "r"(accumulate)
        : "memory");
}

__device__ __forceinline__ void umma_commit(uint64_t *bar)
{
    asm volatile("tcgen05.commit.cta_group::1.mbarrier::arrive::one.shared::cluster.b64 [%0];" ::"r"(smem_u32(bar))
                 : "memory");
}

__device__ __forceinline__ void tc_fence_before() { asm volatile("tcgen05.fence::before_thread_sync;" ::: "memory"); }
__device__ __forceinline__ void tc_fence_after() { asm volatile("tcgen05.fence::after_thread_sync;" ::: "memory"); }

// 32 consecutive accumulator columns of this thread's lane.
__device__ __forceinline__ void tmem_ld32(uint32_t taddr, float (&v)[32])
{
    uint32_t r[32];
    asm volatile(
        "tcgen05.ld.sync.aligned.32x32b.x32.b32 {%0, %1, %2, %3, %4, %5, %6, %7, %8, %9, %10, %11, %12, %13, %14, "
        "%15, %16, %17, %18, %19, %20, %21, %22, %23, %24, %25, %26, %27, %28, %29, %30, %31}, [%32];"
        : "=r"(r[0]), "=r"(r[1]), "=r"(r[2]), "=r"(r[3]), "=r"(r[4]), "=r"(r[5]), "=r"(r[6]), "=r"(r[7]),
          "=r"(r[8]), "=r"(r[9]), "=r"(r[10]), "=r"(r[11]), "=r"(r[12]), "=r"(r[13]), "=r"(r[14]), "=r"(r[15]),
          "=r"(r[16]), "=r"(r[17]), "=r"(r[18]), "=r"(r[19]), "=r"(r[20]), "=r"(r[21]), "=r"(r[22]), "=r"(r[23]),
          "=r"(r[24]), "=r"(r[25]), "=r"(r[26]), "=r"(r[27]), "=r"(r[28]), "=r"(r[29]), "=r"(r[30]), "=r"(r[31])
        : "r"(taddr));
#pragma unroll
    for (int i = 0; i < 32; ++i) v[i] = __uint_as_float(r[i]);
}
__device__ __forceinline__ float tmem_ld1(uint32_t taddr)
{
    uint32_t r;
    asm volatile("tcgen05.ld.sync.aligned.32x32b.x1.b32 {%0}, [%1];" : "=r"(r) : "r"(taddr));
    return __uint_as_float(r);
}
__device__ __forceinline__ void tmem_wait_ld() { asm volatile("tcgen05.wait::ld.sync.aligned;" ::: "memory"); }

// bfloat16 parts of two values: hi = RN(x), lo = RN(x - hi), packed (a in bits 0-15).
__device__ __forceinline__ void split_bf16x2(float a, float b, uint32_t &hi, uint32_t &lo)
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float2 hf = __bfloat1622float2(h);
    const __nv_bfloat162 l = __floats2bfloat162_rn(a - hf.x, b - hf.y);
    hi = *reinterpret_cast<const uint32_t *>(&h);
    lo = *reinterpret_cast<const uint32_t *>(&l);
}

// Raw samples j0 .. j0+7 (j0 a multiple of 8) of the row at element offset off; 0 at or past W.
__device__ __forceinline__ void load8(const LoadParams &L, long long off, int j0, float (&v)[8])
{
    if (L.vec && L.input_type == TK_INPUT_U16) {
        const uint4 q = __ldg(reinterpret_cast<const uint4 *>(static_cast<const uint16_t *>(L.in) + off + j0));
        const uint32_t w[4] = {q.x, q.y, q.z, q.w};
#pragma unroll
        for (int e = 0; e < 4; ++e) {  // count c as (2^23 + c) - 2^23: exact, no integer-to-float conversion
            v[2 * e] = __uint_as_float(0x4B000000u | (w[e] & 0xffffu)) - 8388608.f;
            v[2 * e + 1] = __uint_as_float(0x4B000000u | (w[e] >> 16)) - 8388608.f;
        }
    } else if (L.vec) {
        const float4 *src = reinterpret_cast<const float4 *>(static_cast<const float *>(L.in) + off + j0);
        const float4 a = __ldg(src), b = (j0 + 4 < L.W) ? __ldg(src + 1) : make_float4(0.f, 0.f, 0.f, 0.f);
        v[0] = a.x, v[1] = a.y, v[2] = a.z, v[3] = a.w, v[4] = b.x, v[5] = b.y, v[6] = b.z, v[7] = b.w;
    } else {
#pragma unroll
        for (int e = 0; e < 8; ++e) v[e] = (j0 + e < L.W) ? load_raw(L, off, j0 + e) : 0.f;
    }
#pragma unroll
    for (int e = 0; e < 8; ++e)
        if (j0 + e >= L.W) v[e] = 0.f;
}

// 16-byte asynchronous copy global -> shared (L2 only), and its groups.
__device__ __forceinline__ void cp_async16(uint32_t dst, const void *src)
{
    asm volatile("cp.async.cg.shared.global [%0], [%1], 16;" ::"r"(dst), "l"(src) : "memory");
}
__device__ __forceinline__ void cp_async_commit() { asm volatile("cp.async.commit_group;" ::: "memory"); }
__device__ __forceinline__ void cp_async_wait_prior() { asm volatile("cp.async.wait_group 1;" ::: "memory"); }

// Raw-run staging of the producers (rows 16-byte aligned): per stage, item and
// 16-byte half, one 16-byte slot per producer thread (consecutive threads on
// consecutive slots), two stages.
constexpr int kToepRawBytes = 2 * 4 * 2 * kToepProdWarps * 32 * 16;

// Output row index of detector row gr = b H + r (frame groups: frame b at b/fgrp*fstride + b%fgrp).
__device__ __forceinline__ long long frame_row(const ToepParams &P, long long gr, int &r)
{
    const int H = P.L.H;
    const long long b = gr / H;
    r = (int)(gr - b * H);
    const long long bf = P.fgrp > 0 ? b / P.fgrp * P.fstride + b % P.fgrp : b;
    return bf * H + r;
}

template <int MODE>
__global__ void __launch_bounds__(kToepThreads, 1) filter_toeplitz_kernel(const __grid_constant__ ToepParams P)
{
    extern __shared__ __align__(1024) unsigned char smem[];
    const int R = P.R, mt = P.mt, nk = P.nk, S = P.slots, W = P.L.W;
    const uint32_t slot_part = (uint32_t)R * 128u;  // one bfloat16 part of a 64-column chunk
    unsigned char *hank_hi = smem;
    unsigned char *hank_lo = hank_hi + (size_t)P.ncores * 128;
    unsigned char *ring = hank_lo + (size_t)P.ncores * 128;  // slot s: hi at s*2*slot_part, lo after it
    float *stage = reinterpret_cast<float *>(ring + (size_t)S * 2 * slot_part);
    uint64_t *bars = reinterpret_cast<uint64_t *>(stage + 2 * 33 * kToepPitch);  // a staging buffer per set
    // full/empty per ring slot (up to 8), accf/acce per accumulator buffer (2), drain
    uint64_t *full = bars, *empty = bars + 8, *accf = bars + 16, *acce = bars + 18, *drain = bars + 20;
    volatile int *s_abort = reinterpret_cast<volatile int *>(bars + 21);
    uint32_t *s_tmem = reinterpret_cast<uint32_t *>(bars + 21) + 1;
    unsigned char *raw = reinterpret_cast<unsigned char *>(
        (reinterpret_cast<uintptr_t>(bars + 22) + 127) & ~static_cast<uintptr_t>(127));  // kToepRawBytes

    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    // Hankel cores of T: core s, row rr, element cc holds K[8 s + rr + cc - (Wk - 1)] (K even)
    for (int e = tid; e < P.ncores * 64; e += blockDim.x) {
        const int s = e >> 6, rr = (e >> 3) & 7, cc = e & 7;
        const int m = abs(8 * s + rr + cc - (P.Wk - 1));
        const uint32_t hl = m <= P.kmax ? P.khl[m] : 0u;
        reinterpret_cast<uint16_t *>(hank_hi)[e] = (uint16_t)(hl & 0xffffu);
        reinterpret_cast<uint16_t *>(hank_lo)[e] = (uint16_t)(hl >> 16);
    }
    if (tid == 0) {
        for (int s = 0; s < S; ++s) {
            mbar_init(&full[s], kToepProdWarps * 32);
            mbar_init(&empty[s], 1);
        }
        for (int b = 0; b < 2; ++b) {
            mbar_init(&accf[b], 1);
            mbar_init(&acce[b], kToepEpiWarps * 32);
        }
        mbar_init(drain, 1);
        *s_abort = 0;
        fence_mbar_init();
    }
    if (warp == kToepProdWarps + kToepEpiWarps) {  // the MMA warp owns the tensor memory
        asm volatile("tcgen05.alloc.cta_group::1.sync.aligned.shared::cta.b32 [%0], %1;" ::"r"(smem_u32(s_tmem)),
                     "r"(P.tmem_cols)
                     : "memory");
        asm volatile("tcgen05.relinquish_alloc_permit.cta_group::1.sync.aligned;" ::: "memory");
    }
    fence_proxy_async_smem();  // the Hankel cores are read by the tensor cores
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    const uint32_t tmem = *s_tmem;
    const float sigma = P.q_scale ? *P.q_scale : 1.f;

    if (warp < kToepProdWarps && P.L.vec) {
        // ---------------------------------------------------------------- producers (aligned rows)
        // As below, with each thread's runs of a group of four items copied into shared memory
        // asynchronously one group ahead (cp.async), so that the global-load latency overlaps the
        // conversion of the previous group.  Units u of a tile: chunk u / ngroups, group u % ngroups.
        const int pt = tid;
        constexpr int kMaxItems = 8;
        const int nitems = R / 32, g8 = pt & 7, ngroups = (nitems + 3) / 4, nunits = nk * ngroups;
        const bool f32in = P.L.input_type != TK_INPUT_U16;
        const int esz = f32in ? 4 : 2;
        auto slot16 = [&](int st, int m, int h) -> unsigned char * {
            return raw + ((size_t)(((st * 4 + m) * 2 + h) * (kToepProdWarps * 32) + pt) << 4);
        };
        uint32_t cnt = 0;
        for (long long tile = blockIdx.x; tile < P.ntiles && !*s_abort; tile += gridDim.x) {
            const long long row0 = tile * (R - 1);
            long long off[kMaxItems];
            int rq[kMaxItems];
#pragma unroll
            for (int m = 0; m < kMaxItems; ++m) {
                const long long gr = row0 + (pt >> 3) + 32 * m;
                rq[m] = -1;
                off[m] = 0;
                if (m < nitems && gr < P.nrows) {
                    int r, rr;
                    off[m] = in_row_offset(P.L, frame_row(P, gr, r), rr);
                    rq[m] = r;
                }
            }
            auto issue = [&](int u) {
                const int kc = u / ngroups, g = u - kc * ngroups, st = u & 1;
                const int j0 = P.Wk - 8 - (kc * 64 + g8 * 8);
                if (j0 >= W) return;  // the run lies past the row: zeros, nothing to copy
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    const int r = g ? rq[4 + m] : rq[m];
                    if (r < 0) continue;
                    const char *src = static_cast<const char *>(P.L.in) + ((g ? off[4 + m] : off[m]) + j0) * esz;
                    cp_async16(smem_u32(slot16(st, m, 0)), src);
                    if (f32in && j0 + 4 < W) cp_async16(smem_u32(slot16(st, m, 1)), src + 16);
                }
            };
            issue(0);
            cp_async_commit();
            for (int u = 0; u < nunits; ++u) {
                const int kc = u / ngroups, g = u - kc * ngroups, st = u & 1;
                if (u + 1 < nunits) issue(u + 1);
                cp_async_commit();
                cp_async_wait_prior();  // this unit's copies have landed
                const int slot = (int)(cnt % (uint32_t)S);
                if (g == 0 && cnt >= (uint32_t)S && !mbar_wait_bounded(&empty[slot], ((cnt / S) - 1) & 1u, kWaitLimitNs)) {
                    atomicOr(P.err, ERR_WAIT_TIMEOUT);
                    *s_abort = 1;
                }
                if (*s_abort) break;
                unsigned char *hi = ring + (size_t)slot * 2 * slot_part, *lo = hi + slot_part;
                const int j0 = P.Wk - 8 - (kc * 64 + g8 * 8);
#pragma unroll
                for (int m = 0; m < 4; ++m) {
                    if (4 * g + m >= nitems) break;
                    const int r = g ? rq[4 + m] : rq[m];
                    float v[8];
#pragma unroll
                    for (int e = 0; e < 8; ++e) v[e] = 0.f;
                    if (r >= 0 && j0 < W) {
                        const uint4 a = *reinterpret_cast<const uint4 *>(slot16(st, m, 0));
                        if (!f32in) {
                            const uint32_t w4[4] = {a.x, a.y, a.z, a.w};
#pragma unroll
                            for (int e = 0; e < 4; ++e) {  // count c as (2^23 + c) - 2^23: exact
                                v[2 * e] = __uint_as_float(0x4B000000u | (w4[e] & 0xffffu)) - 8388608.f;
                                v[2 * e + 1] = __uint_as_float(0x4B000000u | (w4[e] >> 16)) - 8388608.f;
                            }
                        } else {
                            v[0] = __uint_as_float(a.x), v[1] = __uint_as_float(a.y);
                            v[2] = __uint_as_float(a.z), v[3] = __uint_as_float(a.w);
                            if (j0 + 4 < W) {
                                const uint4 b2 = *reinterpret_cast<const uint4 *>(slot16(st, m, 1));
                                v[4] = __uint_as_float(b2.x), v[5] = __uint_as_float(b2.y);
                                v[6] = __uint_as_float(b2.z), v[7] = __uint_as_float(b2.w);
                            }
                        }
                        const float rt = weight_row_term(P.L, r);
#pragma unroll
                        for (int e = 0; e < 8; ++e) v[e] = (j0 + e < W) ? pre_from_raw(P.L, r, j0 + e, v[e], rt) : 0.f;
                    }
                    // core row: element cc holds column j0 + 7 - cc (the reversed K order)
                    uint4 h, l;
                    split_bf16x2(v[7], v[6], h.x, l.x);
                    split_bf16x2(v[5], v[4], h.y, l.y);
                    split_bf16x2(v[3], v[2], h.z, l.z);
                    split_bf16x2(v[1], v[0], h.w, l.w);
                    const int i = (pt >> 3) + 32 * (4 * g + m);
                    const uint32_t o = (uint32_t)(i >> 3) * 1024u + (uint32_t)g8 * 128u + (uint32_t)(i & 7) * 16u;
                    *reinterpret_cast<uint4 *>(hi + o) = h;
                    *reinterpret_cast<uint4 *>(lo + o) = l;
                }
                if (g == ngroups - 1) {
                    fence_proxy_async_smem();
                    mbar_arrive(&full[slot]);
                    ++cnt;
                }
            }
            asm volatile("cp.async.wait_all;" ::: "memory");  // nothing in flight into the staging
        }
    } else if (warp < kToepProdWarps) {
        // ---------------------------------------------------------------- producers
        const int pt = tid;  // 0 .. 255
        // A thread's items of a chunk are rows (pt >> 3) + 32 m, m < R/32, at column group pt & 7:
        // the same rows in every chunk of a tile, so their input offsets are formed once per tile.
        constexpr int kMaxItems = 8;  // R <= 256
        const int nitems = R / 32, g8 = pt & 7;
        uint32_t cnt = 0;
        for (long long tile = blockIdx.x; tile < P.ntiles && !*s_abort; tile += gridDim.x) {
            const long long row0 = tile * (R - 1);
            long long off[kMaxItems];
            int rq[kMaxItems];
#pragma unroll
            for (int m = 0; m < kMaxItems; ++m) {
                const long long gr = row0 + (pt >> 3) + 32 * m;
                rq[m] = -1;
                off[m] = 0;
                if (m < nitems && gr < P.nrows) {
                    int r, rr;
                    off[m] = in_row_offset(P.L, frame_row(P, gr, r), rr);
                    rq[m] = r;
                }
            }
            for (int kc = 0; kc < nk; ++kc, ++cnt) {
                const int slot = (int)(cnt % (uint32_t)S);
                if (cnt >= (uint32_t)S && !mbar_wait_bounded(&empty[slot], ((cnt / S) - 1) & 1u, kWaitLimitNs)) {
                    atomicOr(P.err, ERR_WAIT_TIMEOUT);
                    *s_abort = 1;
                }
                if (*s_abort) break;
                unsigned char *hi = ring + (size_t)slot * 2 * slot_part, *lo = hi + slot_part;
                const int j0 = P.Wk - 8 - (kc * 64 + g8 * 8);
                // in groups of four items whose loads are all issued before any is processed
#pragma unroll
                for (int m0 = 0; m0 < kMaxItems; m0 += 4) {
                    if (m0 >= nitems) break;
                    float v[4][8];
#pragma unroll
                    for (int m = 0; m < 4; ++m) {
#pragma unroll
                        for (int e = 0; e < 8; ++e) v[m][e] = 0.f;
                        if (rq[m0 + m] >= 0 && j0 < W) load8(P.L, off[m0 + m], j0, v[m]);
                    }
#pragma unroll
                    for (int m = 0; m < 4; ++m) {
                        if (m0 + m >= nitems) break;
                        const int r = rq[m0 + m];
                        if (r >= 0 && j0 < W) {
                            const float rt = weight_row_term(P.L, r);
#pragma unroll
                            for (int e = 0; e < 8; ++e)
                                if (j0 + e < W) v[m][e] = pre_from_raw(P.L, r, j0 + e, v[m][e], rt);
                        }
                        // core row: element cc holds column j0 + 7 - cc (the reversed K order)
                        uint4 h, l;
                        split_bf16x2(v[m][7], v[m][6], h.x, l.x);
                        split_bf16x2(v[m][5], v[m][4], h.y, l.y);
                        split_bf16x2(v[m][3], v[m][2], h.z, l.z);
                        split_bf16x2(v[m][1], v[m][0], h.w, l.w);
                        const int i = (pt >> 3) + 32 * (m0 + m);
                        const uint32_t o = (uint32_t)(i >> 3) * 1024u + (uint32_t)g8 * 128u + (uint32_t)(i & 7) * 16u;
                        *reinterpret_cast<uint4 *>(hi + o) = h;
                        *reinterpret_cast<uint4 *>(lo + o) = l;
                    }
                }
                fence_proxy_async_smem();
                mbar_arrive(&full[slot]);
            }
        }
    } else if (warp < kToepProdWarps + kToepEpiWarps) {
        // ---------------------------------------------------------------- epilogue
        // Per 32-row chunk of a column tile: warp q loads its TMEM lane quarter (output columns
        // 32 q .. 32 q + 31, one per thread, 33 rows), and the chunk is staged in shared memory
        // (with the next column tile's first column, which warp 0 reads); then thread (q, lane)
        // writes rows q + 4 k of columns 4 lane .. 4 lane + 3: each warp store covers consecutive
        // columns of one row.
        const int q = warp & 3;  // TMEM lane quarter
        const int set = (warp - kToepProdWarps) >> 2;  // chunks of this set's parity, its own staging
        float *stg = stage + set * 33 * kToepPitch;
        int ci = 0;
        const int H = P.L.H;
        uint32_t it = 0;
        for (long long tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x, ++it) {
            // accumulator buffer it & 1, its (it >> 1)-th use
            if (!mbar_wait_bounded(&accf[it & 1u], (it >> 1) & 1u, kWaitLimitNs)) {
                atomicOr(P.err, ERR_WAIT_TIMEOUT);
                *s_abort = 1;
            }
            if (*s_abort) break;
            tc_fence_after();
            const long long row0 = tile * (R - 1);
            for (int m = 0; m < mt; ++m) {
                for (int i0 = 0; i0 < R - 1; i0 += 32) {
                    if ((ci++ & 1) != set) continue;
                    const uint32_t tq = tmem + ((uint32_t)(32 * q) << 16) + (it & 1u) * (uint32_t)(mt * R);
                    const int ilast = min(i0 + 32, R - 1);
                    {
                        float v[32];
                        tmem_ld32(tq + (uint32_t)(m * R + i0), v);
                        const float v32 = tmem_ld1(tq + (uint32_t)(m * R + ilast));
                        tmem_wait_ld();
                        const bool cin = 128 * m + 32 * q + lane < W;
#pragma unroll
                        for (int i = 0; i < 32; ++i) stg[i * kToepPitch + 32 * q + lane] = cin ? v[i] * sigma : 0.f;
                        stg[32 * kToepPitch + 32 * q + lane] = cin ? v32 * sigma : 0.f;
                    }
                    if (q == 0) {  // the next column tile's first column (warp-uniform loads)
                        const bool nt = m + 1 < mt;
                        float t[32], t32 = 0.f;
                        if (nt) {
                            tmem_ld32(tq + (uint32_t)((m + 1) * R + i0), t);
                            t32 = tmem_ld1(tq + (uint32_t)((m + 1) * R + ilast));
                            tmem_wait_ld();
                        }
                        if (lane == 0) {
                            const bool nin = nt && 128 * (m + 1) < W;
#pragma unroll
                            for (int i = 0; i < 32; ++i) stg[i * kToepPitch + 128] = nin ? t[i] * sigma : 0.f;
                            stg[32 * kToepPitch + 128] = nin ? t32 * sigma : 0.f;
                        }
                    }
                    asm volatile("bar.sync %0, 128;" ::"r"(1 + set) : "memory");
                    const int cl = 4 * lane, c0 = 128 * m + cl;
                    if (c0 < W) {
                        // detector row r of frame b for row i0 + q (one division), then stepped by 4
                        long long b = (row0 + i0 + q) / H;
                        int r = (int)(row0 + i0 + q - b * H);
#pragma unroll
                        for (int k = 0; k < 8; ++k) {
                            const int i = q + 4 * k;
                            if (i0 + i < R - 1 && row0 + i0 + i < P.nrows) {
                                const long long bf = P.fgrp > 0 ? b / P.fgrp * P.fstride + b % P.fgrp : b;
                                const long long orow = bf * H + r;
                                const float4 a4 = *reinterpret_cast<const float4 *>(stg + i * kToepPitch + cl);
                                if (MODE == TK_F32) {
                                    *reinterpret_cast<float4 *>(static_cast<float *>(P.out) + orow * P.pitch + c0) = a4;
                                } else {
                                    const float a[5] = {a4.x, a4.y, a4.z, a4.w, stg[i * kToepPitch + cl + 4]};
                                    float bb[5] = {0.f, 0.f, 0.f, 0.f, 0.f};
                                    if (r < H - 1) {  // the next detector row (0 below the last one)
                                        const float4 b4 =
                                            *reinterpret_cast<const float4 *>(stg + (i + 1) * kToepPitch + cl);
                                        bb[0] = b4.x, bb[1] = b4.y, bb[2] = b4.z, bb[3] = b4.w;
                                        bb[4] = stg[(i + 1) * kToepPitch + cl + 4];
                                    }
                                    const size_t base = (size_t)orow * P.pitch;
                                    emit_coef_pair<MODE>(P.out, base, c0, W, a, bb);
                                    if (c0 + 2 < W) emit_coef_pair<MODE>(P.out, base, c0 + 2, W, a + 2, bb + 2);
                                }
                            }
                            r += 4;
                            while (r >= H) {
                                r -= H;
                                ++b;
                            }
                        }
                    }
                    asm volatile("bar.sync %0, 128;" ::"r"(1 + set) : "memory");  // the staging is rewritten next
                }
            }
            tc_fence_before();
            mbar_arrive(&acce[it & 1u]);
        }
    } else if (warp == kToepProdWarps + kToepEpiWarps) {
        // ---------------------------------------------------------------- MMA issue (one lane)
        if (lane == 0) {
            const uint32_t hhi = smem_u32(hank_hi), hlo = smem_u32(hank_lo), rbase = smem_u32(ring);
            uint32_t cnt = 0, it = 0;
            bool issued_any = false;
            for (long long tile = blockIdx.x; tile < P.ntiles; tile += gridDim.x, ++it) {
                // two accumulator buffers: tile it waits only for the epilogue of tile it - 2
                if (it > 1 && !mbar_wait_bounded(&acce[it & 1u], ((it >> 1) - 1) & 1u, kWaitLimitNs)) {
                    atomicOr(P.err, ERR_WAIT_TIMEOUT);
                    *s_abort = 1;
                }
                if (*s_abort) break;
                tc_fence_after();
                for (int kc = 0; kc < nk; ++kc, ++cnt) {
                    const int slot = (int)(cnt % (uint32_t)S);
                    if (!mbar_wait_bounded(&full[slot], (cnt / S) & 1u, kWaitLimitNs)) {
                        atomicOr(P.err, ERR_WAIT_TIMEOUT);
                        *s_abort = 1;
                    }
                    if (*s_abort) break;
                    tc_fence_after();
                    const uint32_t ghi = rbase + (uint32_t)slot * 2u * slot_part, glo = ghi + slot_part;
#pragma unroll 1
                    for (int ks = 0; ks < 4; ++ks) {
                        // G: N = R rows x 16 columns at core column 2 ks (cores along K 128 B apart, row groups 1 KB)
                        const uint64_t bh = umma_desc(ghi + (uint32_t)ks * 256u, 128u, 1024u);
                        const uint64_t bl = umma_desc(glo + (uint32_t)ks * 256u, 128u, 1024u);
                        for (int m = 0; m < mt; ++m) {
                            // T: 128 output columns from core 16 m, K columns from core 8 kc + 2 ks (Hankel)
                            const uint32_t core = (uint32_t)(16 * m + 8 * kc + 2 * ks) * 128u;
                            const uint64_t ah = umma_desc(hhi + core, 128u, 128u);
                            const uint64_t al = umma_desc(hlo + core, 128u, 128u);
                            const uint32_t d = tmem + (it & 1u) * (uint32_t)(mt * R) + (uint32_t)(m * R);
                            umma_bf16(d, ah, bh, P.idesc, (kc > 0 || ks > 0) ? 1u : 0u);
                            umma_bf16(d, ah, bl, P.idesc, 1u);
                            umma_bf16(d, al, bh, P.idesc, 1u);
                            issued_any = true;
                        }
                    }
                    umma_commit(&empty[slot]);  // the slot is free once these MMAs have read it
                }
                if (*s_abort) break;
                umma_commit(&accf[it & 1u]);
            }
            if (issued_any) {  // every MMA has completed before the tensor memory is released
                umma_commit(drain);
                mbar_wait_bounded(drain, 0, kWaitLimitNs);
            }
        }
        __syncwarp();
    }
    tc_fence_before();
    __syncthreads();
    tc_fence_after();
    if (warp == kToepProdWarps + kToepEpiWarps)
        asm volatile("tcgen05.dealloc.cta_group::1.sync.aligned.b32 %0, %1;" ::"r"(tmem), "r"(P.tmem_cols)
                     : "memory");
}

// ---------------------------------------------------------------------------
// host

static uint16_t bf16_rn(double x)
{
    const float f = (float)x;
    uint32_t u;
    std::memcpy(&u, &f, 4);
    if ((u & 0x7fffffffu) > 0x7f800000u) return 0x7fc0;  // NaN
    u += 0x7fffu + ((u >> 16) & 1u);                      // round to nearest even
    return (uint16_t)(u >> 16);
}
static double bf16_value(uint16_t h)
{
    const uint32_t u = (uint32_t)h << 16;
    float f;
    std::memcpy(&f, &u, 4);
    return f;
}

bool toeplitz_supported(int W, int precision, int out_layout)
{
    return W >= 8 && W <= kToepMaxW && out_layout == TK_LAYOUT_PROJECTION && valid_precision(precision);
}

int launch_filter_toeplitz(const LoadParams &L, const float *Hf, int p, void *d_q, int precision,
                           const float *d_q_scale, long long nrows, int pitch, int fgrp, int fstride,
                           cudaStream_t stream)
{
    TK_CHECK(toeplitz_supported(L.W, precision, TK_LAYOUT_PROJECTION), TK_ERR_UNSUPPORTED,
             "filter: the tensor-core Toeplitz form supports 8 <= W <= %d (W = %d)", kToepMaxW, L.W);
    static thread_local ToepParams P;
    std::memset(&P, 0, sizeof(P));
    P.L = L;
    P.out = d_q;
    P.q_scale = (precision == TK_F16 || precision == TK_BF16) ? d_q_scale : nullptr;
    P.err = device_error_word();
    TK_CHECK(P.err, TK_ERR_CUDA, "device error word unavailable");
    P.nrows = nrows;
    P.precision = precision;
    P.pitch = pitch;
    P.fgrp = fgrp > 0 ? fgrp : 0;
    P.fstride = fgrp > 0 ? fstride : 0;
    const int W = L.W;
    P.Wk = (W + 63) / 64 * 64;
    P.nk = P.Wk / 64;
    P.mt = (W + 127) / 128;
    // rows per tile: two accumulators of mt x R columns in the 512 of tensor memory (R a multiple of
    // 32: the producers' row groups)
    static const int kRows[5] = {0, 128, 128, 64, 64};
    P.R = kRows[P.mt];
    P.slots = P.R >= 128 ? 3 : 5;
    P.ncores = 16 * P.mt + P.Wk / 8;
    P.kmax = std::max(P.Wk - 1, 128 * P.mt + 7);
    TK_CHECK(P.kmax <= kToepKmax, TK_ERR_UNSUPPORTED, "filter: Toeplitz kernel table too short");
    P.ntiles = (nrows + P.R - 2) / (P.R - 1);
    uint32_t cols = 32;
    while (cols < (uint32_t)(2 * P.mt * P.R)) cols <<= 1;
    P.tmem_cols = cols;
    // kind::f16 descriptor: D F32 (bits 4-5 = 1), A and B BF16 (bits 7-9, 10-12 = 1), both K-major,
    // N >> 3 at bits 17-22, M >> 4 at bits 24-28
    P.idesc = (1u << 4) | (1u << 7) | (1u << 10) | ((uint32_t)(P.R >> 3) << 17) | ((uint32_t)(128 >> 4) << 24);
    // spatial kernel of the float spectrum (the FFT filter's unnormalised inverse), FP64, split hi/lo;
    // cached per (p, kmax, spectrum bytes): the sum costs about p kmax / 2 table terms, milliseconds
    // at W = 512, which small filter launches would otherwise wait for on the host
    {
        static std::mutex mu;
        static std::map<std::tuple<int, int, uint64_t>, std::vector<uint32_t>> cache;
        uint64_t hsh = 1469598103934665603ull;  // FNV-1a over the spectrum's bytes
        const unsigned char *hb = reinterpret_cast<const unsigned char *>(Hf);
        for (size_t i = 0; i < (size_t)(p / 2 + 1) * sizeof(float); ++i) hsh = (hsh ^ hb[i]) * 1099511628211ull;
        const auto key = std::make_tuple(p, P.kmax, hsh);
        std::lock_guard<std::mutex> lk(mu);
        auto it = cache.find(key);
        if (it == cache.end()) {
            std::vector<uint32_t> khl(P.kmax + 1);
            std::vector<double> ct(p);
            for (int k = 0; k < p; ++k) ct[k] = std::cos(2.0 * M_PI * k / p);
            for (int m = 0; m <= P.kmax; ++m) {
                double s = (double)Hf[0] + (double)Hf[p / 2] * ((m & 1) ? -1.0 : 1.0);
                for (int k = 1; k < p / 2; ++k) s += 2.0 * (double)Hf[k] * ct[(size_t)k * m & (size_t)(p - 1)];
                const uint16_t hi = bf16_rn(s);
                const uint16_t lo = bf16_rn(s - bf16_value(hi));
                khl[m] = (uint32_t)hi | ((uint32_t)lo << 16);
            }
            it = cache.emplace(key, std::move(khl)).first;
        }
        std::memcpy(P.khl, it->second.data(), it->second.size() * sizeof(uint32_t));
    }
    const size_t smem = 1024 + (size_t)P.ncores * 256 + (size_t)P.slots * 2 * P.R * 128 +
                        (size_t)2 * 33 * kToepPitch * 4 + 22 * 8 + 128 + (L.vec ? kToepRawBytes : 0);
    TK_CHECK(smem <= 227 * 1024, TK_ERR_UNSUPPORTED, "filter: Toeplitz form needs %zu B of shared memory", smem);
    const void *fn = nullptr;
    switch (precision) {
    case TK_F32: fn = reinterpret_cast<const void *>(&filter_toeplitz_kernel<TK_F32>); break;
    case TK_F16: fn = reinterpret_cast<const void *>(&filter_toeplitz_kernel<TK_F16>); break;
    case TK_BF16: fn = reinterpret_cast<const void *>(&filter_toeplitz_kernel<TK_BF16>); break;
    default: fn = reinterpret_cast<const void *>(&filter_toeplitz_kernel<TK_F32_COEF>); break;
    }
    TK_CUDA(cudaFuncSetAttribute(fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0;
    TK_CUDA(cudaGetDevice(&dev));
    TK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    const long long grid = std::min<long long>(P.ntiles, sms);
    void *args[] = {&P};
    TK_CUDA(cudaLaunchKernel(fn, dim3((unsigned)std::max<long long>(grid, 1)), dim3(kToepThreads), args, smem, stream));
    count_launch();
    return TK_OK;
}

}  // namespace tk
