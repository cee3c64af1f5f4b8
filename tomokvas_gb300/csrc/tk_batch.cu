// tk_batch.cu -- many FDK reconstructions of uneven sizes in one persistent
// backprojection launch.
//
// Items (geometry, device input, output volume) are submitted to a tk_batch;
// planning lays out one workspace with every item's coefficient image, angle
// table and a device table of per-item parameters (with each item's TMA
// tensor map in global memory), and splits every volume into TX x TY x TZ
// tile units, larger items first.  A run filters each item (one launch per
// item) and then backprojects all units with ONE persistent launch: CTAs
// (as many as fit on the SMs) take units from a global counter, so small and
// large volumes share the GPU without tails.  Items with the quarter-turn
// symmetry instead get tk_fdk_device's quarter-turn launch, on their filter
// stream beside the persistent kernel (same kernel and bits as per volume).  The mbarrier ring of a CTA
// runs on across units (its phase follows the CTA's running projection
// count).  tk_batch_run can capture the whole run once into a CUDA graph and
// replay it.  tk_batch_autotune times every compiled tile shape of the
// batch's storage format on the batch and keeps the fastest.
//
// The arithmetic per update is the per-volume coefficient-image kernel's
// (tk_bp.cu, FBPConeKernel + fQ3D of Lukas-kV/TomoKvas FBPG/kernel.cu:68-177);
// results equal tk_fdk_device's for the same tile shape.
#include "tk_bp_core.cuh"
#include "tk_common.cuh"
#include "tk_internal.h"

#include <algorithm>
#include <cmath>
#include <cstring>
#include <new>
#include <numeric>
#include <vector>
#include <cudaTypedefs.h>

namespace tk {

struct __align__(64) BatchItem {
    CUtensorMap tmap;     // this item's coefficient image (entries viewed as floats)
    float *vol;           // [Z][Y][X]
    const float *q_scale; // 16-bit storage scale, or null
    const float2 *trig;   // (cos, sin) per projection (kernel.cu:430-441)
    long long slice_stride;
    int X, Y, nz, N;
    int BW, BH;           // staged box (entries)
    int tilesX, ntiles, zchunks;
    int unit0;            // first work unit of this item
    float cX, cZ, D, dX, dY, zoff, scale, Wm1, Hm1, fscale;
    unsigned dirx, diry, dirz;
    float halfW;          // W / 2. (kernel.cu:100 compares in double; W / 2 and the sqrtf result are
                          // exact in FP32, so the FP32 comparison decides the same)
};

template <int TX, int TY, int ALIGN>
__device__ __forceinline__ int2 batch_footprint(const BatchItem &I, float2 cs, int x0, int y0, int z0, int z1)
{
    const int xs[2] = {x0, min(x0 + TX - 1, I.X - 1)};
    const int ys[2] = {y0, min(y0 + TY - 1, I.Y - 1)};
    const float aZ0 = flip(I.scale * ((float)z0 + I.zoff), I.dirz);
    const float aZ1 = flip(I.scale * ((float)z1 + I.zoff), I.dirz);
    float umin = 3.0e38f, vmin = 3.0e38f;
#pragma unroll
    for (int i = 0; i < 2; ++i) {
#pragma unroll
        for (int j = 0; j < 2; ++j) {
            const float aX = flip(I.scale * ((float)xs[i] + I.dX), I.dirx);
            const float aY = flip(I.scale * ((float)ys[j] + I.dY), I.diry);
            const float S = aX * cs.x + aY * cs.y;
            const float T = aY * cs.x - aX * cs.y;
            const float U = I.D / (I.D - S);
            umin = fminf(umin, T * U + I.cX);
            vmin = fminf(vmin, fminf(aZ0 * U + I.cZ, aZ1 * U + I.cZ));
        }
    }
    int bx = (int)floorf(umin) - 1;
    bx &= ~(ALIGN - 1);
    return make_int2(bx, (int)floorf(vmin) - 1);
}

// WALK as in update_cimg: 4 (FP32 interpolation of 16-bit storage) for TK_F16
// and TK_BF16 and 1 (packed FP32) for TK_F32_COEF are the per-volume
// defaults; 3 is the selectable FP16 half-math walk.
template <int PREC, int TX, int TY, int TZ, int STAGES, int MINB, int WALK = 4>
__global__ void __launch_bounds__(TX *TY, MINB)
    bp_batch_kernel(const BatchItem *__restrict__ items, int nitems, int nunits, int *counter, unsigned *err,
                    int maxN, int slot_elems)
{
    constexpr int NT = TX * TY;
    constexpr int ES = Cimg<PREC>::kBytes;
    extern __shared__ __align__(128) unsigned char smem[];
    float2 *trig_s = reinterpret_cast<float2 *>(smem + (size_t)STAGES * slot_elems * ES);
    int2 *boxo = reinterpret_cast<int2 *>(trig_s + maxN);
    uint64_t *full = reinterpret_cast<uint64_t *>(boxo + maxN);
    volatile int *ctl = reinterpret_cast<volatile int *>(full + STAGES);  // [0] unit, [1] abort

    const int tid = threadIdx.x;
    const int tx = tid % TX, ty = tid / TX;
    const uint32_t smem0 = smem_u32(smem);
    if (tid == 0) {
        ctl[1] = 0;
        for (int s = 0; s < STAGES; ++s) mbar_init(&full[s], 1);
        fence_mbar_init();
    }
    uint32_t seq = 0;  // projections consumed by this CTA: slot (seq+b) % STAGES, phase ((seq+b) / STAGES) & 1

    for (;;) {
        __syncthreads();  // the previous unit is done with trig_s, boxo and ctl
        if (tid == 0) ctl[0] = atomicAdd(counter, 1);
        __syncthreads();
        const int u = ctl[0];
        if (u >= nunits) break;
        int lo = 0, hi = nitems - 1;  // the item owning unit u: last with unit0 <= u
        while (lo < hi) {
            const int mid = (lo + hi + 1) >> 1;
            if (items[mid].unit0 <= u) lo = mid;
            else hi = mid - 1;
        }
        const BatchItem &I = items[lo];
        const int local = u - I.unit0;
        const int tile = local % I.ntiles, zci = local / I.ntiles;
        const int2 tc = tile_of(tile, I.tilesX, I.ntiles / I.tilesX);
        const int x0 = tc.x * TX, y0 = tc.y * TY;
        const int nz = I.nz;
        // the z chunks of the per-volume kernel (tk_bp.cu bp_cimg_kernel), so that the results are
        // the same bits: 16-bit storage walks only the slices left in a ragged last chunk; FP32
        // coefficients move the last chunk down to end at nz (partial only for nz < TZ)
        const int zc = zci * TZ;
        const bool partial = PREC != TK_F32_COEF ? zc + TZ > nz : nz < TZ;
        const int z0 = PREC != TK_F32_COEF ? zc : (partial ? 0 : min(zc, nz - TZ));
        const int zlast = partial ? nz - 1 - z0 : TZ - 1;
        const int x = x0 + tx, y = y0 + ty;
        const float aX = flip(I.scale * ((float)x + I.dX), I.dirx);
        const float aY = flip(I.scale * ((float)y + I.dY), I.diry);
        const bool inside = (x < I.X) && (y < I.Y);
        const bool active = inside && (sqrtf(aX * aX + aY * aY) < I.halfW);
        float *vcol = I.vol + (size_t)y * I.X + x;

        if (!__syncthreads_or(active)) {  // tile entirely outside the FOV cylinder
            if (inside)
                for (int z = max(zc - z0, 0); z <= zlast; ++z) vcol[(size_t)(z0 + z) * I.slice_stride] = 0.f;
            continue;
        }
        const int N = I.N;
        for (int b = tid; b < N; b += NT) {
            const float2 cs = I.trig[b];
            trig_s[b] = cs;
            boxo[b] = batch_footprint<TX, TY, Cimg<PREC>::kAlign>(I, cs, x0, y0, z0, z0 + zlast);
        }
        if (tid == 0) prefetch_tensormap(&I.tmap);
        __syncthreads();
        const int BW = I.BW;
        const uint32_t stage_bytes = (uint32_t)(BW * I.BH * ES);
        if (tid == 0) {
            for (int k = 0; k < STAGES && k < N; ++k) {
                const uint32_t slot = (seq + k) % STAGES;
                mbar_arrive_expect_tx(&full[slot], stage_bytes);
                tma_load_3d(smem + (size_t)slot * slot_elems * ES, &I.tmap, boxo[k].x * (ES / 4), boxo[k].y, k,
                            &full[slot]);
            }
        }

        const float aZ0 = flip(I.scale * ((float)z0 + I.zoff), I.dirz);
        const float daZ = flip(I.scale, I.dirz);
        float acc[TZ];
#pragma unroll
        for (int z = 0; z < TZ; ++z) acc[z] = 0.f;
        const float cZ = I.cZ, Hm1 = I.Hm1, Wm1 = I.Wm1, cX = I.cX, D = I.D;
        const int BH = I.BH;
        const uint32_t row_bytes = (uint32_t)BW * ES;
        int b = 0;
        for (; b < N; ++b) {
            const uint32_t slot = (seq + b) % STAGES;
            const uint32_t parity = ((seq + b) / STAGES) & 1u;
            const bool got = mbar_wait_bounded(&full[slot], parity, kWaitLimitNs);
            if (!got) {
                atomicOr(err, ERR_WAIT_TIMEOUT);
                ctl[1] = 1;
            }
            if (active && got) {
                float U, uu;
                column_geometry(aX, aY, trig_s[b], D, cX, U, uu);
                if (uu >= 0.f && uu <= Wm1) {  // kernel.cu:127-128
                    const int bx0 = boxo[b].x, by0 = boxo[b].y;
                    const float fla = __fadd_rd(uu, kMagic);
                    const int col = __float_as_int(fla) - kMagicBits - bx0;
                    const float fu = uu - (fla - kMagic);
                    const float v0 = slice_v(aZ0, U, cZ);
                    const float dv = __fmul_rn(daZ, U);
                    const float vL = fmaf((float)zlast, dv, v0);
                    const float vlo = fminf(v0, vL), vhi = fmaxf(v0, vL);
                    const int rlo = (int)floorf(vlo) - by0, rhi = (int)floorf(vhi) - by0;
                    if (col >= 0 && col < BW && rlo >= 0 && rhi < BH) {
                        const uint32_t sbase = smem0 + slot * (uint32_t)slot_elems * ES + (uint32_t)col * ES -
                                               (uint32_t)(kMagicBits + by0) * row_bytes;
                        const float U2 = __fmul_rn(U, U);
                        const bool all_in = vlo >= 0.f && vhi <= Hm1;
                        if (partial) {
                            if (all_in)
                                update_cimg<PREC, TZ, true, true, WALK>(sbase, row_bytes, v0, dv, fu, U2, Hm1, zlast,
                                                                        acc);
                            else
                                update_cimg<PREC, TZ, false, true, WALK>(sbase, row_bytes, v0, dv, fu, U2, Hm1, zlast,
                                                                         acc);
                        } else {
                            if (all_in)
                                update_cimg<PREC, TZ, true, false, WALK>(sbase, row_bytes, v0, dv, fu, U2, Hm1, zlast,
                                                                           acc);
                            else
                                update_cimg<PREC, TZ, false, false, WALK>(sbase, row_bytes, v0, dv, fu, U2, Hm1,
                                                                            zlast, acc);
                        }
                    } else {
                        atomicOr(err, ERR_BOX_OVERFLOW);
                    }
                }
            }
            __syncthreads();  // every thread is done with this slot
            if (ctl[1]) break;
            if (tid == 0 && b + STAGES < N) {
                mbar_arrive_expect_tx(&full[slot], stage_bytes);
                tma_load_3d(smem + (size_t)slot * slot_elems * ES, &I.tmap, boxo[b + STAGES].x * (ES / 4),
                            boxo[b + STAGES].y, b + STAGES, &full[slot]);
            }
        }
        if (ctl[1]) {
            // Leave no copy in flight into shared memory this CTA gives back.
            if (tid == 0) {
                const int issued = min(N, b + STAGES);
                for (int k = b; k < issued; ++k)
                    mbar_wait_bounded(&full[(seq + k) % STAGES], ((seq + k) / STAGES) & 1u, 100000000ull);
            }
            __syncthreads();
            return;
        }
        seq += (uint32_t)N;

        if (inside) {
            const float fs = I.q_scale ? I.fscale / *I.q_scale : I.fscale;
#pragma unroll
            for (int z = 0; z < TZ; ++z) {
                if (z <= zlast && z0 + z >= zc) vcol[(size_t)(z0 + z) * I.slice_stride] = active ? acc[z] * fs : 0.f;
            }
        }
    }
}

struct BatchVariant {
    const void *fn;
    int precision, TX, TY, TZ, STAGES;
    const char *name;
    int walk;  // update_cimg walk; the autotuner tries the FP32-interpolation walks only
};

#define TK_BATCH_W(P, PN, TX, TY, TZ, ST, MB, WK, WN) \
    {reinterpret_cast<const void *>(&bp_batch_kernel<P, TX, TY, TZ, ST, MB, WK>), P, TX, TY, TZ, ST, \
     "batch<" PN "," #TX "," #TY "," #TZ "," #ST ",occ" #MB WN ">", WK}
#define TK_BATCH(P, PN, TX, TY, TZ, ST, MB) TK_BATCH_W(P, PN, TX, TY, TZ, ST, MB, 4, "")

// The first entry of each storage format is its default, with the tile
// shape of the per-volume default (tk_bp.cu) so that both give the same bits:
// the z walk starts at each chunk's first slice, so results depend on TZ.
static const BatchVariant kBatchVariants[] = {
    TK_BATCH(TK_F16, "f16", 16, 16, 64, 3, 2),
    TK_BATCH(TK_BF16, "bf16", 16, 16, 64, 3, 2),
    TK_BATCH(TK_F32_COEF, "f32c", 16, 16, 64, 2, 2),
    TK_BATCH(TK_F16, "f16", 16, 16, 32, 3, 3),
    TK_BATCH(TK_F16, "f16", 16, 16, 48, 3, 2),
    TK_BATCH(TK_F16, "f16", 16, 16, 64, 2, 2),
    TK_BATCH(TK_F32_COEF, "f32c", 16, 16, 32, 3, 2),
    TK_BATCH_W(TK_F16, "f16", 16, 16, 64, 3, 2, 3, ",h16"),  // the FP16 half-math walk
};
constexpr int kNumBatchVariants = (int)(sizeof(kBatchVariants) / sizeof(kBatchVariants[0]));

static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

}  // namespace tk

using namespace tk;

struct tk_batch {
    struct Input {
        tk_geometry g;
        const void *d_in;
        int input_type, layout, window;
        tk_flatfield ff;
        bool has_ff;
        float *d_vol;
        int filter_form = TK_FILTER_AUTO;  // chosen per item by tk_batch_autotune
        bool quad = false;  // backprojected by the per-volume quarter-turn launch, not the persistent kernel
    };
    std::vector<Input> in;
    int precision = TK_F16;
    int variant = -1;  // kBatchVariants index; -1: the default of the precision
    // plan
    char *ws = nullptr;
    size_t ws_bytes = 0;
    bool planned = false;
    int used_variant = -1, nunits = 0, maxN = 0, slot_elems = 0, grid = 0;
    size_t smem = 0;
    size_t off_scale = 0, off_items = 0, off_trig = 0;
    std::vector<size_t> off_q;
    std::vector<BatchItem> h_items;  // host images of the device tables (kept for the async upload)
    std::vector<float2> h_trig;
    // graph
    cudaStream_t cap = nullptr;
    cudaGraphExec_t gexec = nullptr;
    // the items' filters run on several streams forked from the run's stream (parallel branches
    // of the captured graph): most items are too small to fill the GPU one after another
    std::vector<cudaStream_t> fstreams;
    std::vector<cudaEvent_t> fdone;
    cudaEvent_t fork = nullptr;
    // phase timing of the last eager run (tk_batch_timings): start, filters joined, backprojection done
    cudaEvent_t t_ev[3] = {nullptr, nullptr, nullptr};
    bool timed = false;
};

namespace {

void drop_graph(tk_batch *b)
{
    if (b->gexec) cudaGraphExecDestroy(b->gexec);
    b->gexec = nullptr;
}

int find_variant(int precision, int requested)
{
    if (requested >= 0) return kBatchVariants[requested].precision == precision ? requested : -1;
    for (int i = 0; i < kNumBatchVariants; ++i)
        if (kBatchVariants[i].precision == precision) return i;
    return -1;
}

// Workspace layout: [counter | scales | item table | angle tables | coefficient images].
size_t layout_ws(tk_batch *b)
{
    const size_t n = b->in.size();
    size_t off = 256;  // the unit counter
    b->off_scale = off;
    off += align256(n * sizeof(float));
    b->off_items = off;
    off += align256(n * sizeof(BatchItem));
    b->off_trig = off;
    size_t ntrig = 0;
    for (const auto &it : b->in) ntrig += (size_t)it.g.N;
    off += align256(ntrig * sizeof(float2));
    b->off_q.resize(n);
    for (size_t i = 0; i < n; ++i) {
        b->off_q[i] = off;
        off += align256(filtered_bytes(b->in[i].g, b->precision));
    }
    return off;
}

// Per-item tables and work units for tile-shape variant vi; uploads them on st.
int build_tables(tk_batch *b, int vi, cudaStream_t st)
{
    const BatchVariant &V = kBatchVariants[vi];
    static PFN_cuTensorMapEncodeTiled_v12000 encode = nullptr;
    if (!encode) {
        cudaDriverEntryPointQueryResult q;
        void *p = nullptr;
        if (cudaGetDriverEntryPointByVersion("cuTensorMapEncodeTiled", &p, 12000, cudaEnableDefault, &q) ==
                cudaSuccess &&
            q == cudaDriverEntryPointSuccess)
            encode = reinterpret_cast<PFN_cuTensorMapEncodeTiled_v12000>(p);
    }
    TK_CHECK(encode, TK_ERR_CUDA, "cuTensorMapEncodeTiled is unavailable");
    const int n = (int)b->in.size();
    const int ES = (int)entry_size(b->precision);
    const int align = ES >= 16 ? 1 : 16 / ES;
    const int fpe = ES / 4;
    // larger items first: their units start early and the small ones fill the tail
    std::vector<int> order(n);
    std::iota(order.begin(), order.end(), 0);
    auto cost = [&](int i) { const auto &g = b->in[i].g; return (double)g.X * g.Y * g.Z * g.N; };
    std::stable_sort(order.begin(), order.end(), [&](int a, int c) { return cost(a) > cost(c); });

    b->h_items.assign(n, BatchItem{});
    b->h_trig.clear();
    std::vector<size_t> trig_at(n);
    for (int i = 0; i < n; ++i) {
        trig_at[i] = b->h_trig.size();
        const tk_geometry &g = b->in[i].g;
        std::vector<float> cs(g.N), sn(g.N);
        build_trig(g, cs.data(), sn.data());
        for (int k = 0; k < g.N; ++k) b->h_trig.push_back(make_float2(cs[k], sn[k]));
    }
    int units = 0, maxN = 0, slot = 0;
    for (int r = 0; r < n; ++r) {
        const int i = order[r];
        const tk_geometry &g = b->in[i].g;
        BatchItem &I = b->h_items[r];
        const float zoff = tk_default_zoff(&g);
        // Items with the quarter-turn symmetry get the per-volume quarter-turn launch (the same
        // kernel and bits as tk_fdk_device); they own no unit of the persistent kernel.
        b->in[i].quad = backproject_quarter_ok(g, b->precision, g.Z, zoff);
        if (b->in[i].quad) {
            I.unit0 = units;
            continue;
        }
        int BW, BH;
        if (int rc = bp_box_dims(g, g.Z, zoff, V.TX, V.TY, V.TZ, true, align, &BW, &BH)) return rc;
        TK_CHECK(BW * ES / 4 <= 256, TK_ERR_UNSUPPORTED, "batch item %d: tile footprint of %d entries too wide", i,
                 BW);
        const int pitch = storage_pitch(g.W, b->precision);
        cuuint64_t dims[3] = {(cuuint64_t)g.W * fpe, (cuuint64_t)g.H, (cuuint64_t)g.N};
        cuuint64_t strides[2] = {(cuuint64_t)pitch * ES, (cuuint64_t)pitch * g.H * ES};
        cuuint32_t box[3] = {(cuuint32_t)(BW * fpe), (cuuint32_t)BH, 1};
        cuuint32_t estr[3] = {1, 1, 1};
        CUresult cr = encode(&I.tmap, CU_TENSOR_MAP_DATA_TYPE_FLOAT32, 3, b->ws + b->off_q[i], dims, strides, box,
                             estr, CU_TENSOR_MAP_INTERLEAVE_NONE, CU_TENSOR_MAP_SWIZZLE_NONE,
                             CU_TENSOR_MAP_L2_PROMOTION_L2_256B, CU_TENSOR_MAP_FLOAT_OOB_FILL_NONE);
        TK_CHECK(cr == CUDA_SUCCESS, TK_ERR_CUDA, "batch item %d: cuTensorMapEncodeTiled failed (%d)", i, (int)cr);
        I.vol = b->in[i].d_vol;
        I.q_scale = (b->precision == TK_F16 || b->precision == TK_BF16)
                        ? reinterpret_cast<const float *>(b->ws + b->off_scale) + i
                        : nullptr;
        I.trig = reinterpret_cast<const float2 *>(b->ws + b->off_trig) + trig_at[i];
        I.slice_stride = (long long)g.X * g.Y;
        I.X = g.X;
        I.Y = g.Y;
        I.nz = g.Z;
        I.N = g.N;
        I.BW = BW;
        I.BH = BH;
        I.tilesX = (g.X + V.TX - 1) / V.TX;
        I.ntiles = I.tilesX * ((g.Y + V.TY - 1) / V.TY);
        I.zchunks = (g.Z + V.TZ - 1) / V.TZ;
        I.unit0 = units;
        TK_CHECK((long long)units + (long long)I.ntiles * I.zchunks < (1ll << 30), TK_ERR_UNSUPPORTED,
                 "batch too large");
        units += I.ntiles * I.zchunks;
        I.cX = g.cX;
        I.cZ = g.cZ;
        I.D = g.D;
        I.dX = -g.cx;
        I.dY = -g.cy;
        I.zoff = zoff;
        I.scale = g.scale;
        I.Wm1 = (float)(g.W - 1);
        I.Hm1 = (float)(g.H - 1);
        I.fscale = g.dfi * (1.f / (float)reference_pad_length(g.W));  // kernel.cu:113, 575
        I.dirx = g.dirx ? 0x80000000u : 0u;
        I.diry = g.diry ? 0x80000000u : 0u;
        I.dirz = g.dirz ? 0x80000000u : 0u;
        I.halfW = (float)g.W * 0.5f;
        maxN = std::max(maxN, g.N);
        slot = std::max(slot, (BW * BH + 15) / 16 * 16);
    }
    size_t smem = (size_t)V.STAGES * slot * ES + (size_t)maxN * (sizeof(float2) + sizeof(int2)) +
                  (size_t)V.STAGES * sizeof(uint64_t) + 16;
    TK_CHECK(smem <= 227 * 1024, TK_ERR_UNSUPPORTED, "batch: %zu B of shared memory needed", smem);
    TK_CUDA(cudaFuncSetAttribute(V.fn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)smem));
    int dev = 0, sms = 0, per_sm = 0;
    TK_CUDA(cudaGetDevice(&dev));
    TK_CUDA(cudaDeviceGetAttribute(&sms, cudaDevAttrMultiProcessorCount, dev));
    TK_CUDA(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&per_sm, V.fn, V.TX * V.TY, smem));
    TK_CHECK(per_sm > 0, TK_ERR_UNSUPPORTED, "batch kernel does not fit an SM");
    TK_CUDA(cudaMemcpyAsync(b->ws + b->off_items, b->h_items.data(), (size_t)n * sizeof(BatchItem),
                            cudaMemcpyHostToDevice, st));
    TK_CUDA(cudaMemcpyAsync(b->ws + b->off_trig, b->h_trig.data(), b->h_trig.size() * sizeof(float2),
                            cudaMemcpyHostToDevice, st));
    TK_CUDA(cudaStreamSynchronize(st));  // the host images may change on the next plan
    b->used_variant = vi;
    b->nunits = units;
    b->maxN = maxN;
    b->slot_elems = slot;
    b->smem = smem;
    b->grid = std::max(1, std::min(units, per_sm * sms));
    return TK_OK;
}

// Filters of every item, then the persistent backprojection.
constexpr int kFilterStreams = 8;

int enqueue(tk_batch *b, cudaStream_t st)
{
    const int n = (int)b->in.size();
    float *scales = reinterpret_cast<float *>(b->ws + b->off_scale);
    const int K = std::min(n, kFilterStreams);
    if (!b->fork) TK_CUDA(cudaEventCreateWithFlags(&b->fork, cudaEventDisableTiming));
    while ((int)b->fstreams.size() < K) {
        cudaStream_t s;
        cudaEvent_t e;
        TK_CUDA(cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking));
        TK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        b->fstreams.push_back(s);
        b->fdone.push_back(e);
    }
    // phase events on eager runs only (a captured graph records none)
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    TK_CUDA(cudaStreamIsCapturing(st, &cs));
    const bool timing = cs == cudaStreamCaptureStatusNone;
    if (timing) {
        for (auto &e : b->t_ev)
            if (!e) TK_CUDA(cudaEventCreate(&e));
        TK_CUDA(cudaEventRecord(b->t_ev[0], st));
    }
    b->timed = false;
    // item i's filter chain (storage scale, filter) on stream i mod K; each item writes only its
    // own coefficient image and scale, so the chains are independent
    TK_CUDA(cudaEventRecord(b->fork, st));
    for (int k = 0; k < K; ++k) TK_CUDA(cudaStreamWaitEvent(b->fstreams[k], b->fork, 0));
    for (int i = 0; i < n; ++i) {
        const auto &it = b->in[i];
        if (int rc = launch_filter(it.g, it.d_in, it.input_type, it.layout, it.has_ff ? &it.ff : nullptr, it.window,
                                   b->ws + b->off_q[i], b->precision, scales + i, b->fstreams[i % K], 0, 0,
                                   it.filter_form))
            return rc;
    }
    for (int k = 0; k < K; ++k) {
        TK_CUDA(cudaEventRecord(b->fdone[k], b->fstreams[k]));
        TK_CUDA(cudaStreamWaitEvent(st, b->fdone[k], 0));
    }
    if (timing) TK_CUDA(cudaEventRecord(b->t_ev[1], st));
    // the quarter-turn items' launches follow the filters on their streams, beside the persistent
    // kernel
    bool any_quad = false;
    for (int i = 0; i < n; ++i) {
        const auto &it = b->in[i];
        if (!it.quad) continue;
        any_quad = true;
        if (int rc = launch_backproject(it.g, b->ws + b->off_q[i], b->precision, scales + i, it.g.Z,
                                        tk_default_zoff(&it.g), it.d_vol, 0, b->fstreams[i % K]))
            return rc;
    }
    if (b->nunits > 0) {
        int *counter = reinterpret_cast<int *>(b->ws);
        TK_CUDA(cudaMemsetAsync(counter, 0, sizeof(int), st));
        const BatchVariant &V = kBatchVariants[b->used_variant];
        const BatchItem *items = reinterpret_cast<const BatchItem *>(b->ws + b->off_items);
        unsigned *err = device_error_word();
        TK_CHECK(err, TK_ERR_CUDA, "device error word unavailable");
        int nitems = n, nunits = b->nunits, maxN = b->maxN, slot = b->slot_elems;
        void *args[] = {&items, &nitems, &nunits, &counter, &err, &maxN, &slot};
        TK_CUDA(cudaLaunchKernel(V.fn, dim3((unsigned)b->grid), dim3((unsigned)(V.TX * V.TY)), args, b->smem, st));
        count_launch();
    }
    if (any_quad)
        for (int k = 0; k < K; ++k) {
            TK_CUDA(cudaEventRecord(b->fdone[k], b->fstreams[k]));
            TK_CUDA(cudaStreamWaitEvent(st, b->fdone[k], 0));
        }
    if (timing) {
        TK_CUDA(cudaEventRecord(b->t_ev[2], st));
        b->timed = true;
    }
    return TK_OK;
}

}  // namespace

extern "C" int tk_batch_create(tk_batch **out)
{
    TK_CHECK(out, TK_ERR_INVALID, "tk_batch_create: null output");
    *out = new (std::nothrow) tk_batch();
    TK_CHECK(*out, TK_ERR_OOM, "tk_batch_create: out of host memory");
    return TK_OK;
}

extern "C" void tk_batch_destroy(tk_batch *b)
{
    if (!b) return;
    drop_graph(b);
    for (cudaStream_t s : b->fstreams) {
        cudaStreamSynchronize(s);
        cudaStreamDestroy(s);
    }
    for (cudaEvent_t e : b->fdone) cudaEventDestroy(e);
    for (cudaEvent_t e : b->t_ev)
        if (e) cudaEventDestroy(e);
    if (b->fork) cudaEventDestroy(b->fork);
    if (b->cap) cudaStreamDestroy(b->cap);
    delete b;
}

extern "C" int tk_batch_set_precision(tk_batch *b, int precision)
{
    TK_CHECK(b, TK_ERR_INVALID, "null batch");
    TK_CHECK(precision == TK_F16 || precision == TK_BF16 || precision == TK_F32_COEF, TK_ERR_UNSUPPORTED,
             "batch: storage must be a coefficient image (TK_F16, TK_BF16 or TK_F32_COEF)");
    b->precision = precision;
    b->variant = -1;
    b->planned = false;
    drop_graph(b);
    return TK_OK;
}

extern "C" int tk_batch_submit(tk_batch *b, const tk_geometry *g, const void *d_in, int input_type, int layout,
                               const tk_flatfield *ff, int window, float *d_vol)
{
    TK_CHECK(b, TK_ERR_INVALID, "null batch");
    if (int rc = validate_geometry(g)) return rc;
    TK_CHECK(d_in && d_vol, TK_ERR_INVALID, "batch: null device pointer");
    TK_CHECK(input_type == TK_INPUT_F32 || input_type == TK_INPUT_U16, TK_ERR_INVALID, "bad input type %d",
             input_type);
    TK_CHECK(input_type == TK_INPUT_F32 || ff, TK_ERR_INVALID, "batch: raw input needs flat-field parameters");
    TK_CHECK(layout == TK_LAYOUT_SINOGRAM || layout == TK_LAYOUT_PROJECTION, TK_ERR_INVALID, "bad layout %d",
             layout);
    TK_CHECK(window >= TK_WINDOW_RAMLAK && window <= TK_WINDOW_HANN, TK_ERR_INVALID, "bad window %d", window);
    TK_CHECK(g->W <= 2048 && g->Z >= 1, TK_ERR_UNSUPPORTED, "batch: needs W <= 2048 and Z >= 1");
    tk_batch::Input it{};
    it.g = *g;
    it.d_in = d_in;
    it.input_type = input_type;
    it.layout = layout;
    it.window = window;
    it.has_ff = ff != nullptr;
    if (ff) it.ff = *ff;
    it.d_vol = d_vol;
    b->in.push_back(it);
    b->planned = false;
    drop_graph(b);
    return TK_OK;
}

extern "C" int tk_batch_size(const tk_batch *b) { return b ? (int)b->in.size() : -1; }

extern "C" size_t tk_batch_workspace_bytes(tk_batch *b)
{
    if (!b || b->in.empty()) return 0;
    return layout_ws(b);
}

extern "C" int tk_batch_plan(tk_batch *b, void *d_workspace, size_t workspace_bytes, void *stream)
{
    TK_CHECK(b, TK_ERR_INVALID, "null batch");
    TK_CHECK(!b->in.empty(), TK_ERR_STATE, "batch: nothing submitted");
    const size_t need = layout_ws(b);
    TK_CHECK(d_workspace && workspace_bytes >= need, TK_ERR_INVALID, "batch workspace of %zu B needed, %zu given",
             need, workspace_bytes);
    TK_CHECK((reinterpret_cast<uintptr_t>(d_workspace) & 255) == 0, TK_ERR_INVALID,
             "workspace must be 256-byte aligned");
    const int vi = find_variant(b->precision, b->variant);
    TK_CHECK(vi >= 0, TK_ERR_INVALID, "batch: no kernel variant for this storage format");
    drop_graph(b);
    b->planned = false;
    b->ws = static_cast<char *>(d_workspace);
    b->ws_bytes = workspace_bytes;
    if (int rc = build_tables(b, vi, static_cast<cudaStream_t>(stream))) return rc;
    b->planned = true;
    return TK_OK;
}

extern "C" int tk_batch_run(tk_batch *b, int use_graph, void *stream)
{
    TK_CHECK(b, TK_ERR_INVALID, "null batch");
    TK_CHECK(b->planned, TK_ERR_STATE, "batch: call tk_batch_plan first");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    if (!use_graph) return enqueue(b, st);
    if (!b->gexec) {
        TK_CHECK(device_error_word(), TK_ERR_CUDA, "device error word unavailable");  // looked up outside capture
        if (!b->cap) TK_CUDA(cudaStreamCreateWithFlags(&b->cap, cudaStreamNonBlocking));
        TK_CUDA(cudaStreamBeginCapture(b->cap, cudaStreamCaptureModeThreadLocal));
        const int rc = enqueue(b, b->cap);
        cudaGraph_t graph = nullptr;
        const cudaError_t ec = cudaStreamEndCapture(b->cap, &graph);
        if (rc) {
            if (graph) cudaGraphDestroy(graph);
            return rc;
        }
        TK_CUDA(ec);
        const cudaError_t ei = cudaGraphInstantiate(&b->gexec, graph, 0);
        cudaGraphDestroy(graph);
        TK_CUDA(ei);
    }
    TK_CUDA(cudaGraphLaunch(b->gexec, st));
    return TK_OK;
}

extern "C" int tk_batch_timings(tk_batch *b, float *filter_ms, float *bp_ms)
{
    TK_CHECK(b && filter_ms && bp_ms, TK_ERR_INVALID, "tk_batch_timings: null argument");
    TK_CHECK(b->timed, TK_ERR_STATE, "tk_batch_timings: no eager run since the last plan");
    TK_CUDA(cudaEventSynchronize(b->t_ev[2]));
    TK_CUDA(cudaEventElapsedTime(filter_ms, b->t_ev[0], b->t_ev[1]));
    TK_CUDA(cudaEventElapsedTime(bp_ms, b->t_ev[1], b->t_ev[2]));
    return TK_OK;
}

extern "C" int tk_batch_variant_count(void) { return kNumBatchVariants; }

extern "C" const char *tk_batch_variant_name(int i)
{
    return (i >= 0 && i < kNumBatchVariants) ? kBatchVariants[i].name : "";
}

extern "C" int tk_batch_variant(const tk_batch *b) { return b && b->planned ? b->used_variant : -1; }

extern "C" int tk_batch_select_variant(tk_batch *b, int i)
{
    TK_CHECK(b, TK_ERR_INVALID, "null batch");
    TK_CHECK(i == -1 || (i >= 0 && i < kNumBatchVariants && kBatchVariants[i].precision == b->precision),
             TK_ERR_INVALID, "batch variant %d does not exist for this storage format", i);
    b->variant = i;
    b->planned = false;
    drop_graph(b);
    return TK_OK;
}

extern "C" int tk_batch_autotune(tk_batch *b, void *stream, int *variant_out, float *ms_out)
{
    TK_CHECK(b, TK_ERR_INVALID, "null batch");
    TK_CHECK(b->ws, TK_ERR_STATE, "batch: call tk_batch_plan first");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    cudaEvent_t e0 = nullptr, e1 = nullptr;
    TK_CUDA(cudaEventCreate(&e0));
    TK_CUDA(cudaEventCreate(&e1));
    int rc = TK_OK;
    // the filter form of each item: the FFT or the tensor-core Toeplitz product, whichever runs its
    // filter faster (one warm-up and three timed runs each; items of one width get the same answer
    // up to timing noise)
    {
        float *scales = reinterpret_cast<float *>(b->ws + b->off_scale);
        for (size_t i = 0; i < b->in.size() && rc == TK_OK; ++i) {
            auto &it = b->in[i];
            float best_f = 3.0e38f;
            int best_form = TK_FILTER_FFT;
            for (int form : {TK_FILTER_FFT, TK_FILTER_TOEPLITZ}) {
                if (form == TK_FILTER_TOEPLITZ && !toeplitz_supported(it.g.W, b->precision, TK_LAYOUT_PROJECTION))
                    continue;
                auto run = [&]() {
                    return launch_filter(it.g, it.d_in, it.input_type, it.layout, it.has_ff ? &it.ff : nullptr,
                                         it.window, b->ws + b->off_q[i], b->precision, scales + i, st, 0, 0, form);
                };
                if ((rc = run()) != TK_OK) break;
                if (cudaEventRecord(e0, st) != cudaSuccess) { rc = TK_ERR_CUDA; break; }
                for (int k = 0; k < 3 && rc == TK_OK; ++k) rc = run();
                if (rc) break;
                if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
                    rc = cuda_fail(cudaGetLastError(), "batch filter autotune timing");
                    break;
                }
                float ms = 0.f;
                cudaEventElapsedTime(&ms, e0, e1);
                if (ms < best_f) {
                    best_f = ms;
                    best_form = form;
                }
            }
            it.filter_form = best_form;
        }
    }
    int best = -1;
    float best_ms = 3.0e38f;
    for (int vi = 0; vi < kNumBatchVariants && rc == TK_OK; ++vi) {
        if (kBatchVariants[vi].precision != b->precision || kBatchVariants[vi].walk == 3) continue;
        drop_graph(b);
        b->planned = false;
        if (build_tables(b, vi, st) != TK_OK) continue;  // shape does not fit this batch
        b->planned = true;
        if ((rc = enqueue(b, st)) != TK_OK) break;  // warm-up
        if (cudaEventRecord(e0, st) != cudaSuccess) { rc = TK_ERR_CUDA; break; }
        if ((rc = enqueue(b, st)) != TK_OK) break;
        if ((rc = enqueue(b, st)) != TK_OK) break;
        if (cudaEventRecord(e1, st) != cudaSuccess || cudaEventSynchronize(e1) != cudaSuccess) {
            rc = cuda_fail(cudaGetLastError(), "batch autotune timing");
            break;
        }
        float ms = 0.f;
        cudaEventElapsedTime(&ms, e0, e1);
        ms *= 0.5f;
        if (ms < best_ms) {
            best_ms = ms;
            best = vi;
        }
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    if (rc) return rc;
    TK_CHECK(best >= 0, TK_ERR_UNSUPPORTED, "batch autotune: no variant fits");
    b->variant = best;
    drop_graph(b);
    b->planned = false;
    if (int r = build_tables(b, best, st)) return r;
    b->planned = true;
    if (variant_out) *variant_out = best;
    if (ms_out) *ms_out = best_ms;
    return TK_OK;
}

extern "C" int tk_batch_item_quarter_turn(const tk_batch *b, int i)
{
    if (!b || i < 0 || i >= (int)b->in.size() || !b->planned) return -1;
    return b->in[(size_t)i].quad ? 1 : 0;
}

extern "C" int tk_batch_item_filter_form(const tk_batch *b, int i)
{
    if (!b || i < 0 || i >= (int)b->in.size()) return -1;
    return b->in[(size_t)i].filter_form;
}
