// tk_phantom.cu -- analytic cone-beam line integrals of ellipsoids (synthetic input).
//
// The geometry is the backprojector's (FBPG/kernel.cu:68-177, flat virtual
// detector through the rotation axis): the source of projection b sits at
// D*(cos b, sin b, 0) virtual pixels and detector sample (u, v) at
// T = u - cX, Z = v - cZ on the plane S = 0, i.e. at (-T sin b, T cos b, Z).
// Lengths are converted to cm with the virtual pitch tau.  Each ray's chord
// through every ellipsoid is evaluated from its closest approach point in
// the ellipsoid's normalised frame, which keeps FP32 cancellation small.
#include "tk_common.cuh"
#include "tk_internal.h"

#include <cstring>
#include <vector>

namespace tk {

constexpr int kMaxEllipsoids = 160;
constexpr int kPhantomMaxProj = 2048;

struct PhantomParams {
    float *out;
    int W, N, H, layout;
    float cX, cZ, D, tau;
    int nell;
    float e[kMaxEllipsoids][16];  // centre(3) axes(3) R(9) density(1)
    float2 trig[kPhantomMaxProj];
};

__global__ void __launch_bounds__(128) phantom_kernel(const __grid_constant__ PhantomParams P, int b0)
{
    const int u = blockIdx.x * blockDim.x + threadIdx.x;
    const int r = blockIdx.y;
    const int bl = blockIdx.z;
    const int b = b0 + bl;
    if (u >= P.W) return;
    const float2 cs = P.trig[bl];
    const float tau = P.tau;
    const float src[3] = {P.D * cs.x * tau, P.D * cs.y * tau, 0.f};
    const float T = ((float)u - P.cX) * tau;
    const float Zd = ((float)r - P.cZ) * tau;
    float d[3] = {-T * cs.y - src[0], T * cs.x - src[1], Zd};
    const float inv = rsqrtf(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    d[0] *= inv;
    d[1] *= inv;
    d[2] *= inv;
    float acc = 0.f;
    for (int k = 0; k < P.nell; ++k) {
        const float *e = P.e[k];
        float A[3], B[3];
#pragma unroll
        for (int i = 0; i < 3; ++i) {
            const float *R = e + 6 + 3 * i;
            const float ia = 1.f / e[3 + i];
            A[i] = (R[0] * d[0] + R[1] * d[1] + R[2] * d[2]) * ia;
            B[i] = (R[0] * (src[0] - e[0]) + R[1] * (src[1] - e[1]) + R[2] * (src[2] - e[2])) * ia;
        }
        const float a2 = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
        const float t0 = -(A[0] * B[0] + A[1] * B[1] + A[2] * B[2]) / a2;
        const float m0 = fmaf(A[0], t0, B[0]), m1 = fmaf(A[1], t0, B[1]), m2 = fmaf(A[2], t0, B[2]);
        const float m2s = m0 * m0 + m1 * m1 + m2 * m2;
        if (m2s < 1.f) acc += e[15] * 2.f * sqrtf((1.f - m2s) / a2);
    }
    const size_t idx = P.layout == TK_LAYOUT_SINOGRAM ? ((size_t)r * P.N + b) * P.W + u
                                                      : ((size_t)b * P.H + r) * P.W + u;
    P.out[idx] = acc;
}

int launch_phantom(const tk_geometry &g, const double *ell, int nell, int layout, float *d_out,
                   cudaStream_t stream)
{
    TK_CHECK(g.W > 0 && g.N > 0 && g.H > 0 && g.D > 0 && g.tau > 0, TK_ERR_INVALID, "phantom: bad geometry");
    TK_CHECK(d_out && (nell == 0 || ell), TK_ERR_INVALID, "phantom: null pointer");
    TK_CHECK(nell >= 0 && nell <= kMaxEllipsoids, TK_ERR_UNSUPPORTED, "phantom: at most %d ellipsoids",
             kMaxEllipsoids);
    TK_CHECK(layout == TK_LAYOUT_SINOGRAM || layout == TK_LAYOUT_PROJECTION, TK_ERR_INVALID, "phantom: bad layout");
    TK_CHECK(g.H <= 65535, TK_ERR_UNSUPPORTED, "phantom: H > 65535");
    static thread_local PhantomParams P;
    std::memset(&P, 0, sizeof(P));
    P.out = d_out;
    P.W = g.W;
    P.N = g.N;
    P.H = g.H;
    P.layout = layout;
    P.cX = g.cX;
    P.cZ = g.cZ;
    P.D = g.D;
    P.tau = g.tau;
    P.nell = nell;
    for (int k = 0; k < nell; ++k)
        for (int i = 0; i < 16; ++i) P.e[k][i] = (float)ell[16 * k + i];
    std::vector<float> cs(g.N), sn(g.N);
    build_trig(g, cs.data(), sn.data());
    for (int b0 = 0; b0 < g.N; b0 += kPhantomMaxProj) {
        const int nb = std::min(kPhantomMaxProj, g.N - b0);
        for (int i = 0; i < nb; ++i) P.trig[i] = make_float2(cs[b0 + i], sn[b0 + i]);
        dim3 grid((unsigned)((g.W + 127) / 128), (unsigned)g.H, (unsigned)nb);
        phantom_kernel<<<grid, 128, 0, stream>>>(P, b0);
        count_launch();
        TK_CUDA(cudaGetLastError());
    }
    return TK_OK;
}

}  // namespace tk
