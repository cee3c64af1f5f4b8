// tk_refrun.cpp -- runs the reference's own FDK kernels on the GPU.
//
// TEST INFRASTRUCTURE ONLY: used to generate golden fixtures that pin the
// oracle (tests/golden/make_golden.py).  It never runs in the product path.
//
// oracle/ref_build.py compiles Lukas-kV/TomoKvas FBPG/kernel.cu, where it
// lies, into a fatbin (oracle/_ref/tk_ref_kernels.fatbin).  This loader
// drives those kernels and cuFFT in the order of the reference's engine:
//   Initialize            FBPG/kernel.cu:324-428  (one pitched sinogram block)
//   CalcSinCos            FBPG/kernel.cu:430-477
//   fRBcomma              FBPG/kernel.cu:539-555  (RB_comma3DKernel)
//   fConvolution          FBPG/kernel.cu:557-802  (FillFilter, R2C, AbsKernel,
//                                                  per-row R2C, FiltrationKernel, C2R)
//   CalculateReconstruction FBPG/kernel.cu:804-897 (FBPConeKernel per Z block)
// The two by-value kernel argument structs must have the reference's layout
// (FBPG/kernel.cuh:25-61), so they are declared with the same members here.
#include <cuda.h>
#include <cuda_runtime.h>
#include <cufft.h>

#include <chrono>
#include <cmath>
#include <cstdarg>
#include <cstdio>
#include <cstring>
#include <string>
#include <vector>

namespace {

struct rec_par_t {  // layout of _rec_par, FBPG/kernel.cuh:25-40
    float *dev_reconstruction;
    size_t rec_p;
    size_t rec_X;
    float dX;
    size_t rec_Y;
    float dY;
    size_t rec_Z;
    float dZ;
    int ZBlockSize;
    float rot;
    unsigned int dirX, dirY, dirZ;
    float scale;
};

struct sin_par_t {  // layout of _sin_par, FBPG/kernel.cuh:44-61
    float *dev_sinogram[10];
    size_t sin_in_block;
    float *dev_dsin;
    float *dev_dcos;
    size_t sin_p;
    size_t sin_X;
    float cX;
    size_t sin_Y;
    size_t sin_Z;
    float cZ;
    float delta_f;
    float scaling;
    float distance;
    float sampling;
};

std::string g_msg;

int fail(const char *fmt, ...)
{
    char buf[512];
    va_list ap;
    va_start(ap, fmt);
    vsnprintf(buf, sizeof(buf), fmt, ap);
    va_end(ap);
    g_msg = buf;
    return -1;
}

#define RT(call)                                                                             \
    do {                                                                                     \
        cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) return fail("%s: %s", #call, cudaGetErrorString(e_));         \
    } while (0)
#define DRV(call)                                                                            \
    do {                                                                                     \
        CUresult r_ = (call);                                                                \
        if (r_ != CUDA_SUCCESS) return fail("%s: driver error %d", #call, (int)r_);          \
    } while (0)
#define FFT(call)                                                                            \
    do {                                                                                     \
        cufftResult r_ = (call);                                                             \
        if (r_ != CUFFT_SUCCESS) return fail("%s: cufft error %d", #call, (int)r_);          \
    } while (0)

struct Kernels {
    CUmodule mod = nullptr;
    CUfunction fbp = nullptr, rb = nullptr, abs = nullptr, filt = nullptr;
};

int find_kernels(const char *path, Kernels &k)
{
    DRV(cuModuleLoad(&k.mod, path));
    unsigned n = 0;
    DRV(cuModuleGetFunctionCount(&n, k.mod));
    std::vector<CUfunction> fs(n);
    DRV(cuModuleEnumerateFunctions(fs.data(), n, k.mod));
    for (CUfunction f : fs) {
        const char *name = nullptr;
        DRV(cuFuncGetName(&name, f));
        std::string s(name);
        if (s.find("FBPConeKernel") != std::string::npos) k.fbp = f;
        else if (s.find("RB_comma3DKernel") != std::string::npos) k.rb = f;
        else if (s.find("AbsKernel") != std::string::npos) k.abs = f;
        else if (s.find("FiltrationKernel") != std::string::npos) k.filt = f;
    }
    if (!k.fbp || !k.rb || !k.abs || !k.filt) return fail("reference kernels not found in %s", path);
    return 0;
}

// FilteredBackProjection::RamLak (FBPG/kernel.cu:792-802)
float ramlak(int v, float sm)
{
    if (v == 0) return 1. / (4. * sm * sm);
    if ((v % 2) == 0) return 0.;
    return -1. / (v * v * 3.14159265358979323846 * 3.14159265358979323846 * sm * sm);
}

unsigned blocks(size_t n, unsigned b) { return (unsigned)std::ceil((float)n / b); }

}  // namespace

extern "C" const char *tkref_last_error(void) { return g_msg.c_str(); }

using Clock = std::chrono::steady_clock;
static double ms_since(Clock::time_point t0)
{
    return std::chrono::duration<double, std::milli>(Clock::now() - t0).count();
}

// sino: host [H][N][W]; vol_out: host [Z][Y][X] (slices the reference never
// computes stay 0).  times_ms (optional, 6 entries, wall clock with the
// reference's own device synchronisations): [0] upload (Initialize),
// [1] cosine weight (fRBcomma), [2] filter (fConvolution), [3] backprojection
// kernels (sum of FBPConeKernel CUDA-event times), [4] reconstruction loop
// with its per-block D2H (CalculateReconstruction), [5] total.  Returns 0 on
// success.
extern "C" int tkref_fdk(const char *fatbin, const float *sino, int W, float cX, int N, int H, float cZ, float dfi,
                         float D, float tau, int X, float cx, int Y, float cy, int Z, float cz, float rot, float scale,
                         int dirx, int diry, int dirz, int zb, float *vol_out, float *times_ms)
{
    RT(cudaSetDevice(0));
    RT(cudaFree(nullptr));  // primary context for the driver API calls
    Kernels k;
    if (find_kernels(fatbin, k)) return -1;
    double t_upload = 0, t_weight = 0, t_filter = 0, t_recon = 0;
    float t_bp = 0;
    cudaEvent_t e0, e1;
    RT(cudaEventCreate(&e0));
    RT(cudaEventCreate(&e1));
    const auto t_start = Clock::now();
    auto t0 = Clock::now();

    sin_par_t sing;
    std::memset(&sing, 0, sizeof(sing));
    rec_par_t recn;
    std::memset(&recn, 0, sizeof(recn));
    sing.sin_X = W; sing.sin_Y = N; sing.sin_Z = H;
    sing.delta_f = dfi; sing.distance = D; sing.cX = cX; sing.cZ = cZ; sing.sampling = tau;
    sing.scaling = 1;
    recn.rec_X = X; recn.rec_Y = Y; recn.rec_Z = Z;
    recn.dX = -cx; recn.dY = -cy;
    const float dZ = -cz;
    recn.dZ = dZ;
    recn.rot = rot;
    recn.scale = scale;
    recn.dirX = dirx ? 1u << 31 : 0; recn.dirY = diry ? 1u << 31 : 0; recn.dirZ = dirz ? 1u << 31 : 0;

    // Initialize: all rows in one pitched block
    sing.sin_in_block = (size_t)H;
    RT(cudaMallocPitch((void **)&sing.dev_sinogram[0], &sing.sin_p, W * sizeof(float), (size_t)N * H));
    RT(cudaMemcpy2D(sing.dev_sinogram[0], sing.sin_p, sino, W * sizeof(float), W * sizeof(float), (size_t)N * H,
                    cudaMemcpyHostToDevice));
    float nr_Z = (float)(Z - 1) / (float)zb;
    int nblk = (int)std::ceil(nr_Z);
    float dcorZ = (nblk - nr_Z) * zb / 2;
    RT(cudaMallocPitch((void **)&recn.dev_reconstruction, &recn.rec_p, X * sizeof(float), (size_t)Y * zb));

    RT(cudaDeviceSynchronize());
    t_upload = ms_since(t0);

    // CalcSinCos
    std::vector<float> ds(N), dc(N);
    for (int beta = 0; beta < N; beta++) {
        double beta_rad = beta * sing.delta_f + recn.rot;
        ds[beta] = (float)std::sin(beta_rad);
        dc[beta] = (float)std::cos(beta_rad);
    }
    RT(cudaMalloc((void **)&sing.dev_dsin, N * sizeof(float)));
    RT(cudaMalloc((void **)&sing.dev_dcos, N * sizeof(float)));
    RT(cudaMemcpy(sing.dev_dsin, ds.data(), N * sizeof(float), cudaMemcpyHostToDevice));
    RT(cudaMemcpy(sing.dev_dcos, dc.data(), N * sizeof(float), cudaMemcpyHostToDevice));

    // fRBcomma
    t0 = Clock::now();
    {
        void *args[] = {&sing};
        DRV(cuLaunchKernel(k.rb, blocks(N, 16), blocks(H, 16), 1, 16, 16, 1, 0, nullptr, args, nullptr));
        RT(cudaDeviceSynchronize());
    }
    t_weight = ms_since(t0);

    // fConvolution
    t0 = Clock::now();
    int p = 2;
    while (p < W) p *= 2;
    p *= 2;
    sing.scaling /= p;
    size_t comp = p / 2 + 1;
    std::vector<float> filter(comp * 2, 0.f);
    for (int i = 0; i < W; i++) filter[i] = ramlak(i - W / 2, sing.sampling) / 2;
    cufftComplex *dev_filter = nullptr, *dev_data = nullptr;
    float *dev_abs = nullptr;
    RT(cudaMalloc((void **)&dev_filter, sizeof(cufftComplex) * comp));
    RT(cudaMalloc((void **)&dev_abs, sizeof(float) * comp));
    RT(cudaMemcpy(dev_filter, filter.data(), p * sizeof(float), cudaMemcpyHostToDevice));
    cufftHandle plan;
    FFT(cufftPlan1d(&plan, p, CUFFT_R2C, 1));
    FFT(cufftExecR2C(plan, (cufftReal *)dev_filter, dev_filter));
    cufftDestroy(plan);
    {
        size_t c = comp;
        void *args[] = {&c, &dev_filter, &dev_abs, &sing.sampling};
        DRV(cuLaunchKernel(k.abs, blocks(comp, 16), 1, 1, 16, 1, 1, 0, nullptr, args, nullptr));
        RT(cudaDeviceSynchronize());
    }
    RT(cudaMalloc((void **)&dev_data, sizeof(cufftComplex) * comp * N));
    cufftHandle fwd, inv;
    FFT(cufftPlan1d(&fwd, p, CUFFT_R2C, N));
    FFT(cufftPlan1d(&inv, p, CUFFT_C2R, N));
    for (int n = 0; n < H; n++) {
        float *dev_block = (float *)((char *)sing.dev_sinogram[0] + n * (sing.sin_p * sing.sin_Y));
        RT(cudaMemcpy2D(dev_data, comp * sizeof(cufftComplex), dev_block, sing.sin_p, W * sizeof(float), N,
                        cudaMemcpyDeviceToDevice));
        RT(cudaMemset2D((float *)dev_data + W, comp * sizeof(cufftComplex), 0, sizeof(float) * (2 * comp - W), N));
        FFT(cufftExecR2C(fwd, (cufftReal *)dev_data, dev_data));
        size_t c = comp, ny = (size_t)N;
        void *args[] = {&c, &ny, &dev_data, &dev_abs};
        DRV(cuLaunchKernel(k.filt, blocks(N, 16), 1, 1, 16, 1, 1, 0, nullptr, args, nullptr));
        RT(cudaDeviceSynchronize());
        FFT(cufftExecC2R(inv, dev_data, (cufftReal *)dev_data));
        RT(cudaMemcpy2D(dev_block, sing.sin_p, dev_data, comp * sizeof(cufftComplex), W * sizeof(float), N,
                        cudaMemcpyDeviceToDevice));
    }
    cufftDestroy(fwd);
    cufftDestroy(inv);
    cudaFree(dev_data);
    cudaFree(dev_abs);
    cudaFree(dev_filter);
    RT(cudaDeviceSynchronize());
    t_filter = ms_since(t0);

    // CalculateReconstruction
    std::memset(vol_out, 0, sizeof(float) * (size_t)X * Y * Z);
    t0 = Clock::now();
    recn.ZBlockSize = zb;
    for (int n = 0; n < nblk; n++) {
        recn.dZ = dZ + (n - (float)nblk / 2.) * zb + dcorZ;
        void *args[] = {&recn, &sing};
        RT(cudaEventRecord(e0));
        DRV(cuLaunchKernel(k.fbp, blocks(X, 8), blocks(Y, 8), blocks(zb, 8), 8, 8, 8, 0, nullptr, args, nullptr));
        RT(cudaEventRecord(e1));
        RT(cudaDeviceSynchronize());
        float ms = 0.f;
        RT(cudaEventElapsedTime(&ms, e0, e1));
        t_bp += ms;
        int slices = zb;
        if ((n + 1) * zb > Z) slices = Z - n * zb;
        RT(cudaMemcpy2D(vol_out + (size_t)n * zb * X * Y, X * sizeof(float), recn.dev_reconstruction, recn.rec_p,
                        X * sizeof(float), (size_t)Y * slices, cudaMemcpyDeviceToHost));
    }
    t_recon = ms_since(t0);
    if (times_ms) {
        times_ms[0] = (float)t_upload;
        times_ms[1] = (float)t_weight;
        times_ms[2] = (float)t_filter;
        times_ms[3] = t_bp;
        times_ms[4] = (float)t_recon;
        times_ms[5] = (float)ms_since(t_start);
    }
    cudaEventDestroy(e0);
    cudaEventDestroy(e1);
    cudaFree(recn.dev_reconstruction);
    cudaFree(sing.dev_sinogram[0]);
    cudaFree(sing.dev_dsin);
    cudaFree(sing.dev_dcos);
    cuModuleUnload(k.mod);
    return 0;
}
