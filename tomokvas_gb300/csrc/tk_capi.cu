// tk_capi.cu -- C ABI of the GB300 FDK engine (include/tk_fdk.h).
//
// Stage entry points (device buffers, caller's stream), the whole-FDK device
// entry point, and the handle that mirrors FilteredBackProjection
// (Lukas-kV/TomoKvas FBPG/kernel.cuh:82-151, FBPG/kernel.cu:219-897).
#include "tk_common.cuh"
#include "tk_internal.h"

#include <algorithm>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <new>
#include <string>
#include <mutex>
#include <vector>

namespace tk {

// ---------------------------------------------------------------- errors
static thread_local char g_err[1024] = "";

void set_error(const char *fmt, ...)
{
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(g_err, sizeof(g_err), fmt, ap);
    va_end(ap);
}

int cuda_fail(cudaError_t e, const char *what)
{
    set_error("%s: %s (%s)", what, cudaGetErrorString(e), cudaGetErrorName(e));
    return e == cudaErrorMemoryAllocation ? TK_ERR_OOM : TK_ERR_CUDA;
}

// ---------------------------------------------------------------- geometry
int reference_pad_length(int W)
{
    int p = 2;
    while (p < W) p *= 2;  // kernel.cu:570-573
    return p * 2;
}

int validate_geometry(const tk_geometry *g)
{
    TK_CHECK(g, TK_ERR_INVALID, "geometry is NULL");
    TK_CHECK(g->W > 0 && g->N > 0 && g->H > 0, TK_ERR_INVALID, "sinogram size %dx%dx%d invalid", g->W, g->N,
             g->H);
    TK_CHECK(g->X > 0 && g->Y > 0 && g->Z >= 0, TK_ERR_INVALID, "volume size %dx%dx%d invalid", g->X, g->Y, g->Z);
    TK_CHECK(std::isfinite(g->D) && g->D > 0.f, TK_ERR_INVALID, "distance D must be > 0");
    TK_CHECK(std::isfinite(g->tau) && g->tau > 0.f, TK_ERR_INVALID, "sampling tau must be > 0");
    TK_CHECK(std::isfinite(g->scale) && g->scale != 0.f, TK_ERR_INVALID, "scale must be finite and non-zero");
    TK_CHECK(std::isfinite(g->dfi) && std::isfinite(g->rot) && std::isfinite(g->cX) && std::isfinite(g->cZ) &&
                 std::isfinite(g->cx) && std::isfinite(g->cy) && std::isfinite(g->cz),
             TK_ERR_INVALID, "non-finite geometry parameter");
    TK_CHECK(g->W <= 4096 && g->H <= 65535 && g->N <= (1 << 20), TK_ERR_UNSUPPORTED,
             "sinogram %dx%dx%d beyond supported limits (W<=4096, H<=65535)", g->W, g->N, g->H);
    return TK_OK;
}

// CalcSinCos (kernel.cu:430-441): beta_rad = beta * delta_f + rot is formed
// in float, sin/cos are taken in double and stored as float.
void build_trig(const tk_geometry &g, float *cos_out, float *sin_out, int angle0)
{
    for (int b = 0; b < g.N; ++b) {
        const float bf = (float)(angle0 + b) * g.dfi;
        const double beta_rad = (double)(float)(bf + g.rot);
        cos_out[b] = (float)std::cos(beta_rad);
        sin_out[b] = (float)std::sin(beta_rad);
    }
}

// ------------------------------------------------------- device error word
__device__ unsigned g_device_err;

unsigned *device_error_word()
{
    static std::mutex mu;  // host threads making their first call on a device at once
    static unsigned *addr[64] = {};
    int dev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= 64) return nullptr;
    std::lock_guard<std::mutex> lk(mu);
    if (!addr[dev]) {
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, g_device_err) != cudaSuccess) return nullptr;
        addr[dev] = static_cast<unsigned *>(p);
    }
    return addr[dev];
}

}  // namespace tk

using namespace tk;

// ======================================================================== misc
extern "C" int tk_version(void) { return TK_FDK_ABI_VERSION; }

extern "C" const char *tk_last_error(void) { return tk::g_err; }

extern "C" size_t tk_get_free_mem_info(int gpu)
{
    int prev = 0;
    if (cudaGetDevice(&prev) != cudaSuccess) return 0;
    if (cudaSetDevice(gpu) != cudaSuccess) return 0;
    size_t fr = 0, tot = 0;
    if (cudaMemGetInfo(&fr, &tot) != cudaSuccess) fr = 0;
    cudaSetDevice(prev);
    return fr;
}

extern "C" int tk_pad_length(int W) { return W > 0 ? reference_pad_length(W) : -1; }

extern "C" float tk_default_zoff(const tk_geometry *g)
{
    return g ? (float)(-((double)g->Z - 1.0) / 2.0 - (double)g->cz) : 0.f;
}

// kernel.cu:398-400 and 821: nr_Z = (Z-1)/ZB in float, ceil, dcorZ, and
// recn.dZ = dZ + (n - nr_blocks/2.)*ZB + dcorZ with dZ = -centre_Z.
extern "C" int tk_zblock_offsets(const tk_geometry *g, int zb, float *zoff_out, int cap)
{
    if (!g || zb <= 0) {
        set_error("zblock offsets: bad arguments");
        return -TK_ERR_INVALID;
    }
    const float nr_Z = (float)(g->Z - 1) / (float)zb;
    const int nblk = (int)std::ceil(nr_Z);
    const float dcorZ = (nblk - nr_Z) * zb / 2;
    const float dZ = -g->cz;
    for (int n = 0; n < nblk && n < cap && zoff_out; ++n)
        zoff_out[n] = (float)((double)dZ + (n - (float)nblk / 2.) * zb + (double)dcorZ);
    return nblk < 0 ? 0 : nblk;
}

extern "C" int tk_device_error_flags(unsigned *flags_out, int clear)
{
    unsigned *w = device_error_word();
    TK_CHECK(w, TK_ERR_CUDA, "device error word unavailable");
    TK_CUDA(cudaDeviceSynchronize());
    unsigned v = 0;
    TK_CUDA(cudaMemcpy(&v, w, sizeof(v), cudaMemcpyDeviceToHost));
    if (clear) TK_CUDA(cudaMemset(w, 0, sizeof(unsigned)));
    if (flags_out) *flags_out = v;
    return TK_OK;
}

// ================================================================== stage API
extern "C" int tk_filter_projections(const tk_geometry *g, const void *d_in, int input_type, int layout,
                                     const tk_flatfield *ff, int window, void *d_q, int precision, float *d_q_scale,
                                     void *stream)
{
    if (int rc = validate_geometry(g)) return rc;
    return launch_filter(*g, d_in, input_type, layout, ff, window, d_q, precision, d_q_scale,
                         static_cast<cudaStream_t>(stream));
}

extern "C" int tk_backproject(const tk_geometry *g, const void *d_q, int precision, const float *d_q_scale, int nz,
                              float zoff, float *d_vol, int accumulate, void *stream)
{
    if (int rc = validate_geometry(g)) return rc;
    return launch_backproject(*g, d_q, precision, d_q_scale, nz, zoff, d_vol, accumulate,
                              static_cast<cudaStream_t>(stream));
}

static constexpr size_t kWsHeader = 256;

extern "C" size_t tk_filtered_bytes(const tk_geometry *g, int precision)
{
    if (!g || !valid_precision(precision)) return 0;
    return filtered_bytes(*g, precision);
}

extern "C" size_t tk_fdk_workspace_bytes(const tk_geometry *g, int precision)
{
    if (!g || !valid_precision(precision)) return 0;
    return kWsHeader + filtered_bytes(*g, precision);
}

extern "C" int tk_fdk_device(const tk_geometry *g, const void *d_in, int input_type, int layout,
                             const tk_flatfield *ff, int window, int precision, void *d_workspace,
                             size_t workspace_bytes, float *d_vol, void *stream)
{
    if (int rc = validate_geometry(g)) return rc;
    TK_CHECK(valid_precision(precision), TK_ERR_INVALID, "bad precision %d", precision);
    const size_t need = tk_fdk_workspace_bytes(g, precision);
    TK_CHECK(d_workspace && workspace_bytes >= need, TK_ERR_INVALID, "workspace of %zu B needed, %zu given", need,
             workspace_bytes);
    TK_CHECK((reinterpret_cast<uintptr_t>(d_workspace) & 255) == 0, TK_ERR_INVALID,
             "workspace must be 256-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *d_scale = static_cast<float *>(d_workspace);
    void *d_q = static_cast<char *>(d_workspace) + kWsHeader;
    if (int rc = launch_filter(*g, d_in, input_type, layout, ff, window, d_q, precision, d_scale, st)) return rc;
    return launch_backproject(*g, d_q, precision, d_scale, g->Z, tk_default_zoff(g), d_vol, 0, st);
}

// ---------------------------------------------------------------- out-of-core
static size_t align256(size_t x) { return (x + 255) & ~(size_t)255; }

static size_t input_elem_bytes(int input_type) { return input_type == TK_INPUT_U16 ? 2 : 4; }

extern "C" size_t tk_fdk_stream_workspace_bytes(const tk_geometry *g, int input_type, int precision, int chunk)
{
    if (!g || !valid_precision(precision) || chunk <= 0 || g->N <= 0 || g->H <= 0 || g->W <= 0) return 0;
    if (input_type != TK_INPUT_F32 && input_type != TK_INPUT_U16) return 0;
    tk_geometry gc = *g;
    gc.N = std::min(chunk, g->N);
    const size_t raw = (size_t)gc.N * g->H * g->W * input_elem_bytes(input_type);
    return kWsHeader + 2 * align256(raw) + align256(filtered_bytes(gc, precision));
}

namespace {
// Streams and events of one tk_fdk_stream call, released on every return
// path (release is deferred by the runtime until their work has finished).
struct StreamSet {
    cudaStream_t copy = nullptr;
    cudaEvent_t start = nullptr, copied[2] = {nullptr, nullptr}, consumed[2] = {nullptr, nullptr};
    ~StreamSet()
    {
        for (cudaEvent_t e : {start, copied[0], copied[1], consumed[0], consumed[1]})
            if (e) cudaEventDestroy(e);
        if (copy) cudaStreamDestroy(copy);
    }
};
}  // namespace

extern "C" int tk_fdk_stream(const tk_geometry *g, const void *h_in, int input_type, const tk_flatfield *ff,
                             int window, int precision, int chunk, void *d_workspace, size_t workspace_bytes,
                             float *d_vol, void *stream)
{
    if (int rc = validate_geometry(g)) return rc;
    TK_CHECK(valid_precision(precision), TK_ERR_INVALID, "bad precision %d", precision);
    TK_CHECK(input_type == TK_INPUT_F32 || input_type == TK_INPUT_U16, TK_ERR_INVALID, "bad input type %d",
             input_type);
    TK_CHECK(h_in && d_vol, TK_ERR_INVALID, "stream: null pointer");
    TK_CHECK(chunk > 0, TK_ERR_INVALID, "stream: chunk must be > 0");
    const size_t need = tk_fdk_stream_workspace_bytes(g, input_type, precision, chunk);
    TK_CHECK(d_workspace && workspace_bytes >= need, TK_ERR_INVALID, "workspace of %zu B needed, %zu given", need,
             workspace_bytes);
    TK_CHECK((reinterpret_cast<uintptr_t>(d_workspace) & 255) == 0, TK_ERR_INVALID,
             "workspace must be 256-byte aligned");
    const int C = std::min(chunk, g->N);
    const int nchunks = (g->N + C - 1) / C;
    const size_t frame = (size_t)g->H * g->W * input_elem_bytes(input_type);
    char *ws = static_cast<char *>(d_workspace);
    float *d_scale = reinterpret_cast<float *>(ws);
    char *raw[2] = {ws + kWsHeader, ws + kWsHeader + align256(frame * C)};
    void *d_q = ws + kWsHeader + 2 * align256(frame * C);
    const char *host = static_cast<const char *>(h_in);
    cudaStream_t st = static_cast<cudaStream_t>(stream);

    StreamSet ss;
    TK_CUDA(cudaStreamCreateWithFlags(&ss.copy, cudaStreamNonBlocking));
    TK_CUDA(cudaEventCreateWithFlags(&ss.start, cudaEventDisableTiming));
    for (int i = 0; i < 2; ++i) {
        TK_CUDA(cudaEventCreateWithFlags(&ss.copied[i], cudaEventDisableTiming));
        TK_CUDA(cudaEventCreateWithFlags(&ss.consumed[i], cudaEventDisableTiming));
    }
    // copies start only after the caller's earlier work on `stream` (which may use the workspace)
    TK_CUDA(cudaEventRecord(ss.start, st));
    TK_CUDA(cudaStreamWaitEvent(ss.copy, ss.start, 0));
    const float zoff = tk_default_zoff(g);
    // Quarter-turn chunks (FP16 storage, a scan with the quarter-turn symmetry): chunk k holds the
    // four ranges [k L + q N/4, + len), q = 0..3, L = chunk/4, copied one after another, filtered
    // as one image of 4 len projections and backprojected from that compact image by the
    // quarter-turn kernel.  Otherwise chunk k is projections [k chunk, + chunk).
    const int NQ = g->N / 4;
    const bool quad =
        g->N % 4 == 0 && C >= 4 && backproject_quarter_ok(*g, precision, g->Z, zoff);
    const int L = quad ? C / 4 : 0;
    const int nch = quad ? (NQ + L - 1) / L : nchunks;
    auto qlen_of = [&](int k) { return std::min(L, NQ - k * L); };
    auto copy_chunk = [&](int k) -> int {
        if (quad) {
            const int len = qlen_of(k);
            for (int q = 0; q < 4; ++q)
                TK_CUDA(cudaMemcpyAsync(raw[k & 1] + (size_t)q * len * frame, host + (size_t)(k * L + q * NQ) * frame,
                                        (size_t)len * frame, cudaMemcpyHostToDevice, ss.copy));
        } else {
            const int b0 = k * C, nb = std::min(C, g->N - b0);
            TK_CUDA(cudaMemcpyAsync(raw[k & 1], host + (size_t)b0 * frame, (size_t)nb * frame,
                                    cudaMemcpyHostToDevice, ss.copy));
        }
        TK_CUDA(cudaEventRecord(ss.copied[k & 1], ss.copy));
        return TK_OK;
    };
    if (int rc = copy_chunk(0)) return rc;
    if (nch > 1)
        if (int rc = copy_chunk(1)) return rc;
    for (int k = 0; k < nch; ++k) {
        const int slot = k & 1, b0 = k * C;
        tk_geometry gc = *g;
        gc.N = quad ? 4 * qlen_of(k) : std::min(C, g->N - b0);
        TK_CUDA(cudaStreamWaitEvent(st, ss.copied[slot], 0));
        if (int rc = launch_filter(gc, raw[slot], input_type, TK_LAYOUT_PROJECTION, ff, window, d_q, precision,
                                   d_scale, st))
            return rc;
        TK_CUDA(cudaEventRecord(ss.consumed[slot], st));
        if (quad) {
            if (int rc = launch_backproject_quarter(*g, d_q, precision, d_scale, g->Z, zoff, d_vol, k > 0, st, k * L,
                                                    qlen_of(k), true))
                return rc;
        } else if (int rc = launch_backproject(gc, d_q, precision, d_scale, g->Z, zoff, d_vol, k > 0, st, b0)) {
            return rc;
        }
        if (k + 2 < nch) {
            TK_CUDA(cudaStreamWaitEvent(ss.copy, ss.consumed[slot], 0));  // raw[slot] is free again
            if (int rc = copy_chunk(k + 2)) return rc;
        }
    }
    return TK_OK;
}

// ------------------------------------------------------------- adjoint pair
extern "C" int tk_forward_project(const tk_geometry *g, const float *d_vol, int nz, float zoff, float *d_qbar,
                                  int accumulate, void *stream)
{
    if (int rc = validate_geometry(g)) return rc;
    return launch_forward_project(*g, d_vol, nz, zoff, d_qbar, accumulate, static_cast<cudaStream_t>(stream));
}

extern "C" int tk_filter_transpose(const tk_geometry *g, const float *d_qbar, int window, float *d_pbar, int layout,
                                   void *stream)
{
    if (int rc = validate_geometry(g)) return rc;
    return launch_filter_transpose(*g, d_qbar, window, d_pbar, layout, static_cast<cudaStream_t>(stream));
}

extern "C" int tk_fdk_forward(const tk_geometry *g, const float *d_proj, int layout, int window, void *d_workspace,
                              size_t workspace_bytes, float *d_vol, void *stream)
{
    return tk_fdk_device(g, d_proj, TK_INPUT_F32, layout, nullptr, window, TK_F32, d_workspace, workspace_bytes, d_vol,
                         stream);
}

extern "C" int tk_fdk_backward(const tk_geometry *g, const float *d_vol_grad, int layout, int window,
                               void *d_workspace, size_t workspace_bytes, float *d_proj_grad, void *stream)
{
    if (int rc = validate_geometry(g)) return rc;
    const size_t need = tk_fdk_workspace_bytes(g, TK_F32);
    TK_CHECK(d_workspace && workspace_bytes >= need, TK_ERR_INVALID, "workspace of %zu B needed, %zu given", need,
             workspace_bytes);
    TK_CHECK((reinterpret_cast<uintptr_t>(d_workspace) & 255) == 0, TK_ERR_INVALID,
             "workspace must be 256-byte aligned");
    cudaStream_t st = static_cast<cudaStream_t>(stream);
    float *qbar = reinterpret_cast<float *>(static_cast<char *>(d_workspace) + kWsHeader);
    if (int rc = launch_forward_project(*g, d_vol_grad, g->Z, tk_default_zoff(g), qbar, 0, st)) return rc;
    return launch_filter_transpose(*g, qbar, window, d_proj_grad, layout, st);
}

extern "C" int tk_phantom_project(const tk_geometry *g, const double *ell, int nell, int layout, float *d_out,
                                  void *stream)
{
    TK_CHECK(g, TK_ERR_INVALID, "geometry is NULL");
    return launch_phantom(*g, ell, nell, layout, d_out, static_cast<cudaStream_t>(stream));
}

// ======================================================= handle (engine object)
struct tk_fdk {
    int dev = 0;
    int zb = 16;                                 // size_of_Z_block default (kernel.cu:243)
    long long alloc_limit = 1024ll * 1024 * 1024; // memory_limit default (kernel.cu:244)
    int collecting = 0;
    int show = 0;
    tk_geometry g{};
    bool have_sino = false, have_rec = false;
    const void *host_in = nullptr;
    int input_type = TK_INPUT_F32;
    int layout = TK_LAYOUT_SINOGRAM;
    const float *host_dark = nullptr, *host_flat = nullptr;
    tk_flatfield ff{};
    int window = TK_WINDOW_RAMLAK;
    int precision = TK_F32;
    cudaStream_t stream = nullptr, copy_stream = nullptr;
    bool own_stream = false;
    // device state
    void *d_in = nullptr;
    size_t d_in_cap = 0;
    void *d_ws = nullptr;  // [header | filtered projections]
    size_t d_ws_cap = 0;
    float *d_dark = nullptr, *d_flat = nullptr;
    size_t dfl_cap = 0;
    float *d_block[2] = {nullptr, nullptr};
    size_t block_cap = 0;
    bool initialized = false, filtered = false;
    cudaEvent_t ev[10] = {};
    float t_filter = 0, t_bp = 0, t_h2d = 0, t_d2h = 0;
    // pipelined mode: the volume is reconstructed during initialize, angle chunk by chunk
    int pipeline = 0;
    float *d_vol_full = nullptr;
    size_t vol_cap = 0;
    std::vector<cudaEvent_t> ev_blocks;  // last backprojection of each Z block
    bool reconstructed = false;
    int pipe_zb = 0;   // Z-block size the pipelined volume was built with
    int pipe_split = 0;      // > 0: the last block's first pipe_split slices complete at ev_last_half
    cudaEvent_t ev_last_half = nullptr;
    // odd Z blocks run on a second stream, so one block's launch fills the tail of another's
    cudaStream_t aux_stream = nullptr;
    // quarter-turn schedule: the chunks' filters run on their own stream, beside the first launch
    cudaStream_t filt_stream = nullptr;
    cudaEvent_t ev_filt = nullptr, ev_join = nullptr;
    int in_chunk = 0;  // > 0: sinogram-major input stored as [H][nb][W] blocks of in_chunk angles
};

static void release_device(tk_fdk *h)
{
    cudaFree(h->d_in);
    cudaFree(h->d_ws);
    cudaFree(h->d_dark);
    cudaFree(h->d_flat);
    cudaFree(h->d_block[0]);
    cudaFree(h->d_block[1]);
    h->d_in = h->d_ws = nullptr;
    h->d_dark = h->d_flat = nullptr;
    h->d_block[0] = h->d_block[1] = nullptr;
    h->d_in_cap = h->d_ws_cap = h->dfl_cap = h->block_cap = 0;
    cudaFree(h->d_vol_full);
    h->d_vol_full = nullptr;
    h->vol_cap = 0;
    for (cudaEvent_t e : h->ev_blocks) cudaEventDestroy(e);
    h->ev_blocks.clear();
    if (h->ev_last_half) cudaEventDestroy(h->ev_last_half);
    h->ev_last_half = nullptr;
    if (h->ev_filt) cudaEventDestroy(h->ev_filt);
    if (h->ev_join) cudaEventDestroy(h->ev_join);
    h->ev_filt = h->ev_join = nullptr;
    if (h->aux_stream) {
        cudaStreamSynchronize(h->aux_stream);
        cudaStreamDestroy(h->aux_stream);
    }
    h->aux_stream = nullptr;
    if (h->filt_stream) {
        cudaStreamSynchronize(h->filt_stream);
        cudaStreamDestroy(h->filt_stream);
    }
    h->filt_stream = nullptr;
    h->reconstructed = false;
    h->in_chunk = 0;
}

// A setter called after initialize: the filtered projections and a pipelined volume are stale.
static void invalidate(tk_fdk *h)
{
    h->filtered = false;
    h->reconstructed = false;
}

static int ensure(void **p, size_t *cap, size_t need)
{
    if (*cap >= need && *p) return TK_OK;
    cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    TK_CUDA(cudaMalloc(p, need));
    *cap = need;
    return TK_OK;
}

extern "C" int tk_fdk_create(tk_fdk **out)
{
    TK_CHECK(out, TK_ERR_INVALID, "create: out is NULL");
    *out = new (std::nothrow) tk_fdk();
    TK_CHECK(*out, TK_ERR_OOM, "create: out of host memory");
    return TK_OK;
}

extern "C" void tk_fdk_destroy(tk_fdk *h)
{
    if (!h) return;
    int prev = 0;
    cudaGetDevice(&prev);
    if (h->initialized || h->stream || h->d_ws) {
        cudaSetDevice(h->dev);
        if (h->stream) cudaStreamSynchronize(h->stream);
        if (h->copy_stream) cudaStreamSynchronize(h->copy_stream);
        release_device(h);
        for (auto &e : h->ev)
            if (e) cudaEventDestroy(e);
        if (h->copy_stream) cudaStreamDestroy(h->copy_stream);
        if (h->own_stream && h->stream) cudaStreamDestroy(h->stream);
        cudaSetDevice(prev);
    }
    delete h;
}

#define TK_H(h) TK_CHECK(h, TK_ERR_INVALID, "handle is NULL")

extern "C" int tk_fdk_set_gpu_id(tk_fdk *h, int id)
{
    TK_H(h);
    TK_CHECK(!h->initialized, TK_ERR_STATE, "set_gpu_id after initialize");
    h->dev = id;
    return TK_OK;
}
extern "C" int tk_fdk_set_block_size(tk_fdk *h, int zb)
{
    TK_H(h);
    TK_CHECK(zb > 0, TK_ERR_INVALID, "block size must be > 0");
    h->zb = zb;
    return TK_OK;
}
extern "C" int tk_fdk_set_allocation_limit(tk_fdk *h, long long bytes)
{
    TK_H(h);
    TK_CHECK(bytes > 0, TK_ERR_INVALID, "allocation limit must be > 0");
    h->alloc_limit = bytes;  // recorded; the engine keeps each array in one allocation
    return TK_OK;
}
extern "C" int tk_fdk_set_collecting(tk_fdk *h, int collecting)
{
    TK_H(h);
    h->collecting = collecting ? 1 : 0;
    return TK_OK;
}
extern "C" int tk_fdk_set_show_info(tk_fdk *h, int show)
{
    TK_H(h);
    h->show = show ? 1 : 0;
    return TK_OK;
}
// fShowInfo (kernel.cu:901-913): the device summary on stdout.
extern "C" int tk_fdk_show_info(tk_fdk *h)
{
    TK_H(h);
    cudaDeviceProp p{};
    TK_CUDA(cudaGetDeviceProperties(&p, h->dev));
    const size_t fr = tk_get_free_mem_info(h->dev);
    fprintf(stdout, "\nGPU:\n  CUDA device %s has %d Multi-Processors\n", p.name, p.multiProcessorCount);
    fprintf(stdout, "  Each Multi-Processor has %d threads\n", p.maxThreadsPerMultiProcessor);
    fprintf(stdout, "  Max threads per block %d\n", p.maxThreadsPerBlock);
    fprintf(stdout, "  Max threads per dim x %d\n                      y %d\n                      z %d\n",
            p.maxThreadsDim[0], p.maxThreadsDim[1], p.maxThreadsDim[2]);
    fprintf(stdout, "  Total     RAM         %zuMiB\n\n  Free      RAM         %zuMiB\n\n",
            p.totalGlobalMem / 1024 / 1024, fr / 1024 / 1024);
    fflush(stdout);
    return TK_OK;
}
extern "C" int tk_fdk_set_axis_direction(tk_fdk *h, int x, int y, int z)
{
    TK_H(h);
    // SetAxisDirection only ever sets the masks (kernel.cu:499-507)
    if (x) h->g.dirx = 1;
    if (y) h->g.diry = 1;
    if (z) h->g.dirz = 1;
    return TK_OK;
}
extern "C" int tk_fdk_set_sinogram_properties(tk_fdk *h, const float *sinogram, int W, float cX, int N, int H,
                                              float cZ, float dfi, float D, float tau)
{
    TK_H(h);
    h->host_in = sinogram;
    h->input_type = TK_INPUT_F32;
    h->g.W = W;
    h->g.cX = cX;
    h->g.N = N;
    h->g.H = H;
    h->g.cZ = cZ;
    h->g.dfi = dfi;
    h->g.D = D;
    h->g.tau = tau;
    h->have_sino = true;
    invalidate(h);
    return TK_OK;
}
extern "C" int tk_fdk_set_reconstruction_properties(tk_fdk *h, int X, float cx, int Y, float cy, int Z, float cz,
                                                    float rot)
{
    TK_H(h);
    h->g.X = X;
    h->g.cx = cx;
    h->g.Y = Y;
    h->g.cy = cy;
    h->g.Z = Z;
    h->g.cz = cz;
    h->g.rot = rot;
    if (h->g.scale == 0.f) h->g.scale = 1.f;  // recn.scale default (kernel.cu:237)
    h->have_rec = true;
    invalidate(h);
    return TK_OK;
}
extern "C" int tk_fdk_set_scale_xyz(tk_fdk *h, float scale)
{
    TK_H(h);
    h->g.scale = scale;
    invalidate(h);
    return TK_OK;
}
extern "C" int tk_fdk_set_projections_u16(tk_fdk *h, const uint16_t *raw, int layout, const float *dark_hw,
                                          const float *flat_hw, float dark_value, float flat_value, float A, float B,
                                          int invert, float floor_counts)
{
    TK_H(h);
    TK_CHECK(layout == TK_LAYOUT_SINOGRAM || layout == TK_LAYOUT_PROJECTION, TK_ERR_INVALID, "bad layout");
    TK_CHECK(floor_counts > 0.f, TK_ERR_INVALID, "floor_counts must be > 0");
    TK_CHECK(flat_hw || flat_value > 0.f, TK_ERR_INVALID, "flat field missing");
    h->host_in = raw;
    h->input_type = TK_INPUT_U16;
    h->layout = layout;
    h->host_dark = dark_hw;
    h->host_flat = flat_hw;
    h->ff.dark_value = dark_value;
    h->ff.flat_value = flat_value;
    h->ff.A = A;
    h->ff.B = B;
    h->ff.invert = invert ? 1 : 0;
    h->ff.floor_counts = floor_counts;
    invalidate(h);
    return TK_OK;
}
extern "C" int tk_fdk_set_input_layout(tk_fdk *h, int layout)
{
    TK_H(h);
    TK_CHECK(layout == TK_LAYOUT_SINOGRAM || layout == TK_LAYOUT_PROJECTION, TK_ERR_INVALID, "bad layout");
    h->layout = layout;
    invalidate(h);
    return TK_OK;
}
extern "C" int tk_fdk_set_filter(tk_fdk *h, int window)
{
    TK_H(h);
    TK_CHECK(window >= TK_WINDOW_RAMLAK && window <= TK_WINDOW_HANN, TK_ERR_INVALID, "bad window %d", window);
    h->window = window;
    invalidate(h);
    return TK_OK;
}
extern "C" int tk_fdk_set_precision(tk_fdk *h, int precision)
{
    TK_H(h);
    TK_CHECK(valid_precision(precision), TK_ERR_INVALID, "bad precision %d", precision);
    h->precision = precision;
    invalidate(h);
    return TK_OK;
}
extern "C" int tk_fdk_set_stream(tk_fdk *h, void *stream)
{
    TK_H(h);
    TK_CHECK(!h->initialized, TK_ERR_STATE, "set_stream after initialize");
    h->stream = static_cast<cudaStream_t>(stream);
    h->own_stream = false;
    return TK_OK;
}

extern "C" int tk_fdk_set_pipeline(tk_fdk *h, int on)
{
    TK_H(h);
    h->pipeline = on ? 1 : 0;
    h->reconstructed = false;
    return TK_OK;
}

static int elapsed(cudaEvent_t a, cudaEvent_t b, float *acc)
{
    float ms = 0;
    TK_CUDA(cudaEventElapsedTime(&ms, a, b));
    *acc += ms;
    return TK_OK;
}

// Initialize (kernel.cu:324-428): device, allocations, host->device copy.
extern "C" int tk_fdk_initialize(tk_fdk *h)
{
    TK_H(h);
    TK_CHECK(h->have_sino && h->have_rec, TK_ERR_STATE,
             "initialize before set_sinogram_properties / set_reconstruction_properties");
    if (int rc = validate_geometry(&h->g)) return rc;
    TK_CHECK(h->host_in, TK_ERR_INVALID, "initialize: no projection data");
    TK_CUDA(cudaSetDevice(h->dev));
    if (!h->stream) {
        TK_CUDA(cudaStreamCreateWithFlags(&h->stream, cudaStreamNonBlocking));
        h->own_stream = true;
    }
    if (!h->copy_stream) TK_CUDA(cudaStreamCreateWithFlags(&h->copy_stream, cudaStreamNonBlocking));
    for (auto &e : h->ev)
        if (!e) TK_CUDA(cudaEventCreate(&e));
    const tk_geometry &g = h->g;
    const size_t n = (size_t)g.W * g.N * g.H;
    const size_t in_bytes = n * (h->input_type == TK_INPUT_U16 ? 2 : 4);
    if (int rc = ensure(&h->d_in, &h->d_in_cap, in_bytes)) return rc;
    if (int rc = ensure(&h->d_ws, &h->d_ws_cap, tk_fdk_workspace_bytes(&g, h->precision))) return rc;
    h->t_h2d = h->t_filter = h->t_bp = h->t_d2h = 0;
    TK_CUDA(cudaEventRecord(h->ev[0], h->stream));
    // Input whose storage scale is known before the data is seen (FP32
    // storage, or uint16 with scalar flat/dark) is copied in angle chunks and
    // each chunk is filtered as soon as it has landed, so the upload overlaps
    // the filter; otherwise one copy, and the filter runs later.  Sinogram-major
    // input ([H][N][W]) is packed chunk by chunk into [H][nb][W] blocks by a
    // strided copy, which the filter reads as a sinogram of nb angles.
    const bool scale_free = !(h->precision == TK_F16 || h->precision == TK_BF16) ||
                            (h->input_type == TK_INPUT_U16 && !h->host_dark && !h->host_flat);
    // Pipelined mode (tk_fdk_set_pipeline), with the Z-block schedule into a whole-volume buffer:
    // the projections upload in chunks of N/8; the chunks of the first quarter of the angles are
    // backprojected block by block as they land (this covers the rest of the upload); once every
    // chunk is filtered, each block gets one accumulating launch over the rest, so blocks
    // complete one after another and each block's copy to the host (calculate_reconstruction)
    // overlaps the next block's launch.  The last block's launch is split at a multiple of 64
    // slices (same bits as one launch) so that half of its copy overlaps the other half.  A
    // volume that does not fit beside the projections falls back to the regular path.
    bool pipe = h->pipeline && !h->collecting && scale_free && g.N >= 2 * 64;
    h->reconstructed = false;
    if (pipe) {
        const size_t vbytes = (size_t)g.X * g.Y * std::max(g.Z, 1) * sizeof(float);
        if (h->vol_cap < vbytes || !h->d_vol_full) {
            cudaFree(h->d_vol_full);
            h->d_vol_full = nullptr;
            h->vol_cap = 0;
            if (cudaMalloc(reinterpret_cast<void **>(&h->d_vol_full), vbytes) == cudaSuccess) {
                h->vol_cap = vbytes;
            } else {
                (void)cudaGetLastError();
                h->d_vol_full = nullptr;
                pipe = false;
            }
        }
    }
    const int chunk = pipe ? std::max(32, (g.N + 7) / 8) : 64;
    const int nchunks = (g.N + chunk - 1) / chunk;
    // first quarter of the angles: at 1024^3 its 60 ms of backprojection covers the rest of a slow
    // (25 GB/s) upload, and the three quarters left give the block copies 180 ms to overlap
    const int major_end = std::min(g.N - chunk, chunk * std::max(1, (nchunks + 2) / 4));
    const bool overlap = scale_free && g.N >= 2 * chunk;
    int nblk = 0;
    std::vector<float> zoff;
    if (pipe) {
        if (!h->aux_stream) TK_CUDA(cudaStreamCreateWithFlags(&h->aux_stream, cudaStreamNonBlocking));
        if (!h->ev_filt) TK_CUDA(cudaEventCreateWithFlags(&h->ev_filt, cudaEventDisableTiming));
        if (!h->ev_join) TK_CUDA(cudaEventCreateWithFlags(&h->ev_join, cudaEventDisableTiming));
        nblk = tk_zblock_offsets(&g, h->zb, nullptr, 0);
        zoff.resize((size_t)std::max(nblk, 1));
        tk_zblock_offsets(&g, h->zb, zoff.data(), nblk);
        while ((int)h->ev_blocks.size() < nblk) {
            cudaEvent_t e;
            TK_CUDA(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
            h->ev_blocks.push_back(e);
        }
    }
    // The first-quarter chunks are backprojected in one launch over all blocks when that is the
    // same arithmetic as one launch per block: every slice's coordinate (float)z + zoff[n] equals
    // (float)(n zb + z) + zoff[0], and the blocks start on 64-slice z-chunk boundaries.
    int merged_slices = 0;
    if (pipe && h->zb % 64 == 0) {
        bool same = true;
        for (int n = 0; n < nblk && same; ++n) {
            int slices = h->zb;
            if ((long long)(n + 1) * h->zb > g.Z) slices = g.Z - n * h->zb;
            for (int z = 0; z < slices && same; ++z)
                same = (float)z + zoff[n] == (float)(n * h->zb + z) + zoff[0];
            merged_slices += slices;
        }
        if (!same) merged_slices = 0;
    }
    // Quarter-turn schedule (the FP16 quarter-turn kernel applies to every launch it needs): chunk c
    // holds the four ranges [c qL + k N/4, + qL), qC chunks of N/4 (the first of 8, 6, 5, 4, 3 that
    // divides N/4), filtered on their own stream as they land (detector frames: one launch over
    // the chunk's four ranges as frame groups); once the first qE = (qC + 2) / 4
    // chunks (a quarter to a third of the angles) are filtered, one launch backprojects them while
    // the other chunks land and filter beside it; then one launch per block over the rest.
    int qC = 0, qL = 0, qE = 0;
    if (pipe && g.N % 4 == 0) {
        for (int c : {8, 6, 5, 4, 3})
            if ((g.N / 4) % c == 0) {
                qC = c;
                break;
            }
        bool ok = qC > 0;
        for (int n = 0; n < nblk && ok; ++n) {
            int slices = h->zb;
            if ((long long)(n + 1) * h->zb > g.Z) slices = g.Z - n * h->zb;
            ok = backproject_quarter_ok(g, h->precision, slices, zoff[n]);
            const int split = n == nblk - 1 ? (slices / 2) / 64 * 64 : 0;
            if (ok && split > 0)
                ok = backproject_quarter_ok(g, h->precision, split, zoff[n]) &&
                     backproject_quarter_ok(g, h->precision, slices - split, zoff[n] + (float)split);
        }
        if (ok && merged_slices > 0) ok = backproject_quarter_ok(g, h->precision, merged_slices, zoff[0]);
        if (ok) {
            qL = g.N / 4 / qC;
            qE = (qC + 2) / 4;
            if (!h->filt_stream) TK_CUDA(cudaStreamCreateWithFlags(&h->filt_stream, cudaStreamNonBlocking));
        } else {
            qC = 0;
        }
    }
    h->in_chunk = overlap && h->layout == TK_LAYOUT_SINOGRAM ? (qC > 0 ? qL : chunk) : 0;
    if (!overlap)
        TK_CUDA(cudaMemcpyAsync(h->d_in, h->host_in, in_bytes, cudaMemcpyHostToDevice, h->stream));
    if (h->input_type == TK_INPUT_U16) {
        const size_t fb = (size_t)g.W * g.H * sizeof(float);
        if (h->host_dark || h->host_flat) {
            void *pd = h->d_dark, *pf = h->d_flat;
            size_t cap = h->dfl_cap;
            if (cap < fb) {
                cudaFree(pd);
                cudaFree(pf);
                pd = pf = nullptr;
                TK_CUDA(cudaMalloc(&pd, fb));
                TK_CUDA(cudaMalloc(&pf, fb));
                cap = fb;
            }
            h->d_dark = static_cast<float *>(pd);
            h->d_flat = static_cast<float *>(pf);
            h->dfl_cap = cap;
        }
        h->ff.dark = nullptr;
        h->ff.flat = nullptr;
        if (h->host_dark) {
            TK_CUDA(cudaMemcpyAsync(h->d_dark, h->host_dark, fb, cudaMemcpyHostToDevice, h->stream));
            h->ff.dark = h->d_dark;
        }
        if (h->host_flat) {
            TK_CUDA(cudaMemcpyAsync(h->d_flat, h->host_flat, fb, cudaMemcpyHostToDevice, h->stream));
            h->ff.flat = h->d_flat;
        }
    }
    h->filtered = false;
    if (overlap) {
        // copies on the copy stream (after the flat/dark uploads above), filters on the stream
        TK_CUDA(cudaEventRecord(h->ev[8], h->stream));
        TK_CUDA(cudaStreamWaitEvent(h->copy_stream, h->ev[8], 0));
        const size_t frame = in_bytes / (size_t)g.N;
        float *d_scale = static_cast<float *>(h->d_ws);
        char *d_q = static_cast<char *>(h->d_ws) + kWsHeader;
        const size_t qframe = filtered_bytes(g, h->precision) / (size_t)g.N;
        const size_t slab = (size_t)g.X * g.Y;
        TK_CUDA(cudaEventRecord(h->ev[2], h->stream));
        // The angle ranges of each chunk, in upload order: one contiguous range, or for the
        // quarter-turn schedule the four ranges [c qL + k N/4, + qL), a set that a quarter turn maps
        // onto itself.
        struct Range {
            int a, n;
        };
        std::vector<std::vector<Range>> chunks;
        const int nq = g.N / 4;
        if (qC > 0) {
            for (int c = 0; c < qC; ++c) {
                chunks.emplace_back();
                for (int k = 0; k < 4; ++k) chunks.back().push_back({c * qL + k * nq, qL});
            }
        } else {
            for (int b0 = 0; b0 < g.N; b0 += chunk) chunks.push_back({{b0, std::min(chunk, g.N - b0)}});
        }
        // chunks backprojected as they land (contiguous chunks), or together once the last of them is
        // filtered (quarter-turn chunks)
        const int early = !pipe ? 0 : (qC > 0 ? qE : major_end / chunk);
        cudaStream_t fs = qC > 0 ? h->filt_stream : h->stream;  // the filters' stream
        if (qC > 0) TK_CUDA(cudaStreamWaitEvent(fs, h->ev[8], 0));
        auto bp_early = [&](int c, int nz, float zo, float *vol, int acc, cudaStream_t st) -> int {
            if (qC > 0) return launch_backproject_quarter(g, d_q, h->precision, d_scale, nz, zo, vol, 0, st, 0, qE * qL);
            const Range r = chunks[c][0];
            tk_geometry gc = g;
            gc.N = r.n;
            return launch_backproject(gc, d_q + (size_t)r.a * qframe, h->precision, d_scale, nz, zo, vol, acc, st,
                                      r.a);
        };
        auto bp_rest = [&](int nz, float zo, float *vol, cudaStream_t st) -> int {
            if (qC > 0)
                return launch_backproject_quarter(g, d_q, h->precision, d_scale, nz, zo, vol, 1, st, qE * qL,
                                                  (qC - qE) * qL);
            tk_geometry gr = g;
            gr.N = g.N - major_end;
            return launch_backproject(gr, d_q + (size_t)major_end * qframe, h->precision, d_scale, nz, zo, vol, 1,
                                      st, major_end);
        };
        for (int c = 0; c < (int)chunks.size(); ++c) {
            for (const Range &r : chunks[c]) {
                const size_t off = (size_t)r.a * frame;
                if (h->layout == TK_LAYOUT_PROJECTION) {
                    TK_CUDA(cudaMemcpyAsync(static_cast<char *>(h->d_in) + off,
                                            static_cast<const char *>(h->host_in) + off, (size_t)r.n * frame,
                                            cudaMemcpyHostToDevice, h->copy_stream));
                } else {
                    const size_t row = frame / (size_t)g.H;  // one detector row of one angle
                    TK_CUDA(cudaMemcpy2DAsync(static_cast<char *>(h->d_in) + off, (size_t)r.n * row,
                                              static_cast<const char *>(h->host_in) + (size_t)r.a * row,
                                              (size_t)g.N * row, (size_t)r.n * row, (size_t)g.H,
                                              cudaMemcpyHostToDevice, h->copy_stream));
                }
            }
            TK_CUDA(cudaEventRecord(h->ev[9], h->copy_stream));
            TK_CUDA(cudaStreamWaitEvent(fs, h->ev[9], 0));
            if (qC > 0 && h->layout == TK_LAYOUT_PROJECTION) {  // the chunk's four ranges in one launch
                tk_geometry gc = g;
                gc.N = 4 * qL;
                const size_t a = (size_t)c * qL;
                if (int rc = launch_filter(gc, static_cast<char *>(h->d_in) + a * frame, h->input_type, h->layout,
                                           &h->ff, h->window, d_q + a * qframe, h->precision, d_scale, fs, qL, nq))
                    return rc;
            } else {
                for (const Range &r : chunks[c]) {
                    tk_geometry gc = g;
                    gc.N = r.n;
                    if (int rc = launch_filter(gc, static_cast<char *>(h->d_in) + (size_t)r.a * frame,
                                               h->input_type, h->layout, &h->ff, h->window,
                                               d_q + (size_t)r.a * qframe, h->precision, d_scale, fs))
                        return rc;
                }
            }
            if (qC > 0 && c + 1 != qE) continue;  // the quarter-turn schedule's one early launch follows chunk qE - 1
            if (qC > 0) {
                TK_CUDA(cudaEventRecord(h->ev_filt, fs));
                TK_CUDA(cudaStreamWaitEvent(h->stream, h->ev_filt, 0));
            }
            if (c < early && merged_slices > 0) {
                if (int rc = bp_early(c, merged_slices, zoff[0], h->d_vol_full, c > 0, h->stream)) return rc;
            } else if (c < early) {
                if (nblk > 1) {  // the odd blocks' stream waits for this chunk's filters
                    TK_CUDA(cudaEventRecord(h->ev_filt, h->stream));
                    TK_CUDA(cudaStreamWaitEvent(h->aux_stream, h->ev_filt, 0));
                }
                for (int n = 0; n < nblk; ++n) {
                    int slices = h->zb;
                    if ((long long)(n + 1) * h->zb > g.Z) slices = g.Z - n * h->zb;  // kernel.cu:838-840
                    if (int rc = bp_early(c, slices, zoff[n], h->d_vol_full + (size_t)n * h->zb * slab, c > 0,
                                          (n & 1) ? h->aux_stream : h->stream))
                        return rc;
                }
            }
        }
        h->pipe_split = 0;
        if (pipe) {
            TK_CUDA(cudaEventRecord(h->ev_filt, fs));
            if (qC > 0) TK_CUDA(cudaStreamWaitEvent(h->stream, h->ev_filt, 0));
            if (nblk > 1) TK_CUDA(cudaStreamWaitEvent(h->aux_stream, h->ev_filt, 0));  // the last filter
            for (int n = 0; n < nblk; ++n) {
                int slices = h->zb;
                if ((long long)(n + 1) * h->zb > g.Z) slices = g.Z - n * h->zb;
                float *vb = h->d_vol_full + (size_t)n * h->zb * slab;
                cudaStream_t bs = (n & 1) ? h->aux_stream : h->stream;  // every launch of block n
                const int split = n == nblk - 1 ? (slices / 2) / 64 * 64 : 0;
                if (split > 0) {
                    if (!h->ev_last_half)
                        TK_CUDA(cudaEventCreateWithFlags(&h->ev_last_half, cudaEventDisableTiming));
                    if (int rc = bp_rest(split, zoff[n], vb, bs)) return rc;
                    TK_CUDA(cudaEventRecord(h->ev_last_half, bs));
                    if (int rc = bp_rest(slices - split, zoff[n] + (float)split, vb + (size_t)split * slab, bs))
                        return rc;
                    h->pipe_split = split;
                } else if (int rc = bp_rest(slices, zoff[n], vb, bs)) {
                    return rc;
                }
                TK_CUDA(cudaEventRecord(h->ev_blocks[n], bs));
            }
            if (nblk > 1) {  // later work on the stream sees both streams' launches
                TK_CUDA(cudaEventRecord(h->ev_join, h->aux_stream));
                TK_CUDA(cudaStreamWaitEvent(h->stream, h->ev_join, 0));
            }
        }
        TK_CUDA(cudaEventRecord(h->ev[3], h->stream));
        h->reconstructed = pipe;
        h->pipe_zb = h->zb;
        TK_CUDA(cudaEventRecord(h->ev[1], h->copy_stream));
        TK_CUDA(cudaStreamSynchronize(h->copy_stream));  // the host buffer is only borrowed until we return
        h->filtered = true;
    } else {
        TK_CUDA(cudaEventRecord(h->ev[1], h->stream));
        TK_CUDA(cudaStreamSynchronize(h->stream));  // the host buffer is only borrowed until we return
    }
    if (int rc = elapsed(h->ev[0], h->ev[1], &h->t_h2d)) return rc;
    h->initialized = true;
    if (h->show) fprintf(stdout, "tk_fdk: %zu MiB of projections on GPU %d\n", in_bytes >> 20, h->dev);
    return TK_OK;
}

// Sinogram-major input uploaded in angle chunks lies on the device as [H][nb][W]
// blocks (tk_fdk_initialize); a setter called after initialize needs it
// filtered again as one [H][N][W] sinogram, so it is unpacked first.
static int unpack_input(tk_fdk *h)
{
    if (h->in_chunk <= 0) return TK_OK;
    const tk_geometry &g = h->g;
    const size_t row = (size_t)g.W * (h->input_type == TK_INPUT_U16 ? 2 : 4);
    const size_t bytes = row * g.N * g.H;
    void *flat = nullptr;
    TK_CUDA(cudaMalloc(&flat, bytes));
    for (int b0 = 0; b0 < g.N; b0 += h->in_chunk) {
        const int nb = std::min(h->in_chunk, g.N - b0);
        const cudaError_t e = cudaMemcpy2DAsync(static_cast<char *>(flat) + (size_t)b0 * row, (size_t)g.N * row,
                                                static_cast<const char *>(h->d_in) + (size_t)b0 * row * g.H,
                                                (size_t)nb * row, (size_t)nb * row, (size_t)g.H,
                                                cudaMemcpyDeviceToDevice, h->stream);
        if (e != cudaSuccess) {
            cudaFree(flat);
            TK_CUDA(e);
        }
    }
    TK_CUDA(cudaStreamSynchronize(h->stream));
    cudaFree(h->d_in);
    h->d_in = flat;
    h->d_in_cap = bytes;
    h->in_chunk = 0;
    return TK_OK;
}

static int run_filter(tk_fdk *h)
{
    if (h->filtered) return TK_OK;
    if (int rc = unpack_input(h)) return rc;
    float *d_scale = static_cast<float *>(h->d_ws);
    void *d_q = static_cast<char *>(h->d_ws) + kWsHeader;
    TK_CUDA(cudaEventRecord(h->ev[2], h->stream));
    if (int rc = launch_filter(h->g, h->d_in, h->input_type, h->layout, &h->ff, h->window, d_q, h->precision, d_scale,
                               h->stream))
        return rc;
    TK_CUDA(cudaEventRecord(h->ev[3], h->stream));
    h->filtered = true;
    return TK_OK;
}

static int check_device_flags(cudaStream_t st)
{
    unsigned *w = device_error_word();
    TK_CHECK(w, TK_ERR_CUDA, "device error word unavailable");
    unsigned v = 0;
    TK_CUDA(cudaMemcpyAsync(&v, w, sizeof(v), cudaMemcpyDeviceToHost, st));
    TK_CUDA(cudaStreamSynchronize(st));
    if (v) {
        cudaMemsetAsync(w, 0, sizeof(unsigned), st);
        cudaStreamSynchronize(st);
        set_error("kernel self-check failed (flags 0x%x)", v);
        return TK_ERR_DEVICE;
    }
    return TK_OK;
}

// CalculateReconstruction (kernel.cu:804-897).
extern "C" int tk_fdk_calculate_reconstruction(tk_fdk *h, tk_block_sink sink, void *user)
{
    TK_H(h);
    TK_CHECK(h->initialized, TK_ERR_STATE, "calculate_reconstruction before initialize");
    TK_CHECK(sink, TK_ERR_INVALID, "calculate_reconstruction: sink is NULL");
    TK_CUDA(cudaSetDevice(h->dev));
    const tk_geometry &g = h->g;
    const int zb = h->zb;
    const int nblk = tk_zblock_offsets(&g, zb, nullptr, 0);
    std::vector<float> zoff((size_t)std::max(nblk, 1));
    tk_zblock_offsets(&g, zb, zoff.data(), nblk);
    const size_t slab = (size_t)g.X * g.Y;
    if (h->reconstructed && !h->collecting && h->pipe_zb == zb) {
        // pipelined: the volume was reconstructed during initialize; block n is copied out once its
        // last backprojection has run, and lands before block n+1 is requested from the sink
        cudaEvent_t d2h_done[2] = {h->ev[6], h->ev[7]};
        TK_CUDA(cudaEventRecord(h->ev[4], h->stream));  // every backprojection queued by initialize has run
        float *prev_host = nullptr;
        for (int n = 0; n < nblk; ++n) {
            int slices = zb;
            if ((long long)(n + 1) * zb > g.Z) slices = g.Z - n * zb;  // kernel.cu:838-840
            if (prev_host) TK_CUDA(cudaEventSynchronize(d2h_done[(n - 1) & 1]));
            float *host = sink(user, n, 0);
            TK_CHECK(host, TK_ERR_IO, "block sink returned NULL for block %d", n);
            const float *src = h->d_vol_full + (size_t)n * zb * slab;
            int done = 0;  // slices already queued
            if (n == nblk - 1 && h->pipe_split > 0 && h->pipe_split < slices) {
                TK_CUDA(cudaStreamWaitEvent(h->copy_stream, h->ev_last_half, 0));
                TK_CUDA(cudaMemcpyAsync(host, src, slab * (size_t)h->pipe_split * sizeof(float),
                                        cudaMemcpyDeviceToHost, h->copy_stream));
                done = h->pipe_split;
            }
            TK_CUDA(cudaStreamWaitEvent(h->copy_stream, h->ev_blocks[n], 0));
            TK_CUDA(cudaMemcpyAsync(host + (size_t)done * slab, src + (size_t)done * slab,
                                    slab * (size_t)(slices - done) * sizeof(float), cudaMemcpyDeviceToHost,
                                    h->copy_stream));
            TK_CUDA(cudaEventRecord(d2h_done[n & 1], h->copy_stream));
            prev_host = host;
        }
        TK_CUDA(cudaEventRecord(h->ev[5], h->copy_stream));
        TK_CUDA(cudaStreamSynchronize(h->copy_stream));
        TK_CUDA(cudaStreamSynchronize(h->stream));
        elapsed(h->ev[2], h->ev[3], &h->t_bp);  // filter + backprojection, interleaved by chunk
        elapsed(h->ev[4], h->ev[5], &h->t_d2h);  // the copies' tail after the last backprojection
        return check_device_flags(h->stream);
    }
    const size_t block_bytes = slab * zb * sizeof(float);
    if (h->block_cap < block_bytes || !h->d_block[0]) {
        cudaFree(h->d_block[0]);
        cudaFree(h->d_block[1]);
        h->d_block[0] = h->d_block[1] = nullptr;
        h->block_cap = 0;
        TK_CUDA(cudaMalloc(&h->d_block[0], block_bytes));
        TK_CUDA(cudaMalloc(&h->d_block[1], block_bytes));
        h->block_cap = block_bytes;
    }
    if (int rc = run_filter(h)) return rc;
    const float *d_scale = static_cast<const float *>(h->d_ws);
    const void *d_q = static_cast<const char *>(h->d_ws) + kWsHeader;
    cudaEvent_t bp_done[2] = {h->ev[4], h->ev[5]};
    cudaEvent_t d2h_done[2] = {h->ev[6], h->ev[7]};
    float *prev_host = nullptr;
    for (int n = 0; n < nblk; ++n) {
        const int k = n & 1;
        // slices delivered for this block (kernel.cu:838-840)
        int slices = zb;
        if ((long long)(n + 1) * zb > g.Z) slices = g.Z - n * zb;
        if (n >= 2) TK_CUDA(cudaStreamWaitEvent(h->stream, d2h_done[k], 0));  // block buffer k is free again
        if (!h->collecting) {
            if (int rc = launch_backproject(g, d_q, h->precision, d_scale, slices, zoff[n], h->d_block[k], 0,
                                            h->stream))
                return rc;
            TK_CUDA(cudaEventRecord(bp_done[k], h->stream));
        }
        if (prev_host) TK_CUDA(cudaEventSynchronize(d2h_done[k ^ 1]));  // block n-1 has landed
        float *host = sink(user, n, h->collecting);
        TK_CHECK(host, TK_ERR_IO, "block sink returned NULL for block %d", n);
        const size_t bytes = slab * (size_t)slices * sizeof(float);
        if (h->collecting) {
            // previous partial volume -> device, then vol = new + previous (kernel.cu:849-876)
            TK_CUDA(cudaMemcpyAsync(h->d_block[k], host, bytes, cudaMemcpyHostToDevice, h->stream));
            if (int rc = launch_backproject(g, d_q, h->precision, d_scale, slices, zoff[n], h->d_block[k], 1,
                                            h->stream))
                return rc;
            TK_CUDA(cudaEventRecord(bp_done[k], h->stream));
        }
        TK_CUDA(cudaStreamWaitEvent(h->copy_stream, bp_done[k], 0));
        TK_CUDA(cudaMemcpyAsync(host, h->d_block[k], bytes, cudaMemcpyDeviceToHost, h->copy_stream));
        TK_CUDA(cudaEventRecord(d2h_done[k], h->copy_stream));
        prev_host = host;
    }
    TK_CUDA(cudaStreamSynchronize(h->copy_stream));
    TK_CUDA(cudaStreamSynchronize(h->stream));
    if (h->filtered) elapsed(h->ev[2], h->ev[3], &h->t_filter);
    if (nblk > 0) elapsed(bp_done[(nblk - 1) & 1], d2h_done[(nblk - 1) & 1], &h->t_d2h);  // the last copy's tail
    return check_device_flags(h->stream);
}

extern "C" int tk_fdk_reconstruct_device(tk_fdk *h, float *d_vol)
{
    TK_H(h);
    TK_CHECK(h->initialized, TK_ERR_STATE, "reconstruct_device before initialize");
    TK_CHECK(d_vol, TK_ERR_INVALID, "reconstruct_device: d_vol is NULL");
    TK_CUDA(cudaSetDevice(h->dev));
    const bool was = h->filtered;
    if (int rc = run_filter(h)) return rc;
    const float *d_scale = static_cast<const float *>(h->d_ws);
    const void *d_q = static_cast<const char *>(h->d_ws) + kWsHeader;
    TK_CUDA(cudaEventRecord(h->ev[4], h->stream));
    if (int rc = launch_backproject(h->g, d_q, h->precision, d_scale, h->g.Z, tk_default_zoff(&h->g), d_vol, 0,
                                    h->stream))
        return rc;
    TK_CUDA(cudaEventRecord(h->ev[5], h->stream));
    TK_CUDA(cudaStreamSynchronize(h->stream));
    if (!was) elapsed(h->ev[2], h->ev[3], &h->t_filter);
    elapsed(h->ev[4], h->ev[5], &h->t_bp);
    return check_device_flags(h->stream);
}

extern "C" int tk_fdk_get_timings(tk_fdk *h, float *filter_ms, float *bp_ms, float *h2d_ms, float *d2h_ms)
{
    TK_H(h);
    if (filter_ms) *filter_ms = h->t_filter;
    if (bp_ms) *bp_ms = h->t_bp;
    if (h2d_ms) *h2d_ms = h->t_h2d;
    if (d2h_ms) *d2h_ms = h->t_d2h;
    return TK_OK;
}
