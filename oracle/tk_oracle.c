/*
 * tk_oracle.c -- CPU oracle for the FDK cone-beam hot path.
 *
 * TEST INFRASTRUCTURE ONLY: tests/, __graft_entry__.smoke() (as the checker)
 * and bench.py's CPU-baseline leg use it.  The shipped library never links,
 * loads or calls it.
 *
 * Pinned against the reference itself: tests/golden/ref_*.npz hold outputs of
 * the reference's own FBPG/kernel.cu kernels with cuFFT on a GB300
 * (oracle/ref_build.py, oracle/tk_refrun.cpp, tests/golden/make_golden.py);
 * tests/test_golden_reference.py checks both restatements against them, and
 * tests/test_oracle.py adds closed-form consequences of the reference's code.
 *
 * Every function below restates one step of the reference
 * (Lukas-kV/TomoKvas, FBPG/kernel.cu and FBPG/rsq_load.cpp); the reference
 * line each one follows is cited beside it.  Build with -ffp-contract=off so
 * x86 and aarch64 hosts round identically.
 */
#include "tk_oracle.h"

#include <math.h>
#include <pthread.h>
#include <stdlib.h>
#include <string.h>

#define ORC_PI 3.14159265358979323846

int orc_version(void) { return 3; }

/* ------------------------------------------------------------------------ */
/* tiny parallel-for over [0, n) with dynamic chunks (pthreads, no OpenMP)   */

typedef void (*orc_body)(void *ctx, long i);
typedef struct {
    long n, chunk;
    long next; /* accessed with __atomic builtins */
    orc_body fn;
    void *ctx;
} orc_pool;

static void *orc_worker(void *arg)
{
    orc_pool *p = (orc_pool *)arg;
    for (;;) {
        long s = __atomic_fetch_add(&p->next, p->chunk, __ATOMIC_RELAXED);
        if (s >= p->n) break;
        long e = s + p->chunk < p->n ? s + p->chunk : p->n;
        for (long i = s; i < e; ++i) p->fn(p->ctx, i);
    }
    return NULL;
}

static void orc_parallel_for(long n, int nthreads, orc_body fn, void *ctx)
{
    if (n <= 0) return;
    if (nthreads < 1) nthreads = 1;
    if (nthreads > 256) nthreads = 256;
    if ((long)nthreads > n) nthreads = (int)n;
    orc_pool p;
    p.n = n;
    p.chunk = n / ((long)nthreads * 16) + 1;
    p.next = 0;
    p.fn = fn;
    p.ctx = ctx;
    if (nthreads == 1) {
        orc_worker(&p);
        return;
    }
    pthread_t th[256];
    int started = 0;
    for (int t = 1; t < nthreads; ++t)
        if (pthread_create(&th[started], NULL, orc_worker, &p) == 0) ++started;
    orc_worker(&p);
    for (int t = 0; t < started; ++t) pthread_join(th[t], NULL);
}

/* ------------------------------------------------------------------------ */
/* radix-2 complex FFT (own implementation), float and double flavours       */

static int orc_log2i(int n)
{
    int l = 0;
    while ((1 << l) < n) ++l;
    return l;
}

/* forward (sign=-1) or unnormalised inverse (sign=+1) transform in place.
 * tw: p/2 twiddles exp(-2 pi i k / p) (re, im interleaved). */
#define ORC_FFT_BODY(T)                                                         \
    int lg = orc_log2i(n);                                                     \
    for (int i = 0, j = 0; i < n; ++i) {                                       \
        if (i < j) {                                                           \
            T tr = re[i], ti = im[i];                                          \
            re[i] = re[j]; im[i] = im[j];                                      \
            re[j] = tr; im[j] = ti;                                            \
        }                                                                      \
        int m = n >> 1;                                                        \
        while (m >= 1 && (j & m)) { j ^= m; m >>= 1; }                         \
        j |= m;                                                                \
    }                                                                          \
    for (int s = 1; s <= lg; ++s) {                                            \
        int half = 1 << (s - 1), step = n >> s;                                \
        for (int k = 0; k < n; k += 2 * half) {                                \
            for (int j = 0; j < half; ++j) {                                   \
                T wr = tw[2 * (j * step)], wi = tw[2 * (j * step) + 1];        \
                if (sign > 0) wi = -wi;                                        \
                int a = k + j, b = a + half;                                   \
                T xr = re[b] * wr - im[b] * wi;                                \
                T xi = re[b] * wi + im[b] * wr;                                \
                re[b] = re[a] - xr; im[b] = im[a] - xi;                        \
                re[a] = re[a] + xr; im[a] = im[a] + xi;                        \
            }                                                                  \
        }                                                                      \
    }

static void orc_fft_f32(float *re, float *im, int n, const float *tw, int sign) { ORC_FFT_BODY(float) }
static void orc_fft_f64(double *re, double *im, int n, const double *tw, int sign) { ORC_FFT_BODY(double) }

static void orc_twiddles_f64(double *tw, int n)
{
    for (int k = 0; k < n / 2; ++k) {
        double a = -2.0 * ORC_PI * (double)k / (double)n;
        tw[2 * k] = cos(a);
        tw[2 * k + 1] = sin(a);
    }
}

/* ------------------------------------------------------------------------ */
/* filter construction                                                       */

/* kernel.cu:570-573: p = 2; while (p < W) p *= 2; p *= 2; */
int orc_pad_length(int W)
{
    int p = 2;
    while (p < W) p *= 2;
    return p * 2;
}

/* FilteredBackProjection::RamLak, kernel.cu:792-802 (returns float). */
static float orc_ramlak(int v, float sm)
{
    if (v == 0) return (float)(1. / (4. * sm * sm));
    if ((v % 2) == 0) return 0.f;
    return (float)(-1. / (v * v * ORC_PI * ORC_PI * sm * sm));
}

/* Frequency windows applied to the reference spectrum, k = 0..p/2. */
static double orc_window(int window, int k, int p)
{
    double f = (double)k / (double)p; /* cycles per sample, 0..0.5 */
    if (window == ORC_WIN_SHEPP_LOGAN) {
        if (k == 0) return 1.0;
        double x = ORC_PI * f;
        return sin(x) / x;
    }
    if (window == ORC_WIN_HANN) return 0.5 * (1.0 + cos(2.0 * ORC_PI * f));
    return 1.0;
}

/* Spectrum Hf[k] = tau |R2C_p(h)[k]| * window, k = 0..p/2, computed in double
 * from the float taps of FillFilter (kernel.cu:783-790, 620-646). */
static void orc_spectrum_f64(int W, double tau, int window, int p, double *Hf)
{
    float *h = (float *)calloc((size_t)p, sizeof(float));
    for (int i = 0; i < W; ++i) h[i] = orc_ramlak(i - W / 2, (float)tau) / 2;
    double *ct = (double *)malloc(sizeof(double) * (size_t)p);
    double *st = (double *)malloc(sizeof(double) * (size_t)p);
    for (int m = 0; m < p; ++m) {
        double a = 2.0 * ORC_PI * (double)m / (double)p;
        ct[m] = cos(a);
        st[m] = sin(a);
    }
    for (int k = 0; k <= p / 2; ++k) {
        double sr = 0, si = 0;
        for (int i = 0; i < W; ++i) {
            int m = (int)(((long)k * i) % p);
            sr += h[i] * ct[m];
            si -= h[i] * st[m];
        }
        Hf[k] = tau * sqrt(sr * sr + si * si) * orc_window(window, k, p);
    }
    free(h); free(ct); free(st);
}

int orc_filter_kernel_f64(int W, double tau, int window, int p, double *k_out)
{
    if (W < 2 || tau <= 0) return -1;
    if (p <= 0) p = orc_pad_length(W);
    if (p < 2 * W || (p & (p - 1))) return -1;
    double *Hf = (double *)malloc(sizeof(double) * (size_t)(p / 2 + 1));
    orc_spectrum_f64(W, tau, window, p, Hf);
    /* k[n] = (1/p) sum_{k=0}^{p-1} Hf_full[k] cos(2 pi k n / p) */
    for (int n = -(W - 1); n <= W - 1; ++n) {
        double s = Hf[0] + Hf[p / 2] * ((n & 1) ? -1.0 : 1.0);
        for (int k = 1; k < p / 2; ++k) {
            long m = ((long)k * (long)(n < 0 ? -n : n)) % p;
            s += 2.0 * Hf[k] * cos(2.0 * ORC_PI * (double)m / (double)p);
        }
        k_out[n + W - 1] = s / (double)p;
    }
    free(Hf);
    return p;
}

/* ------------------------------------------------------------------------ */
/* Z blocking (kernel.cu:398-400 and 819-821)                                */

int orc_zblocks(const orc_geom *g, float *zoff_out, int cap)
{
    int zb = g->zb > 0 ? g->zb : 16;
    float nr_Z = (float)(g->Z - 1) / (float)zb;
    int nblk = (int)ceilf(nr_Z);
    float dcorZ = (nblk - nr_Z) * zb / 2;
    float dZ = -g->cz;
    for (int n = 0; n < nblk && n < cap; ++n)
        zoff_out[n] = (float)((double)dZ + (n - (float)nblk / 2.) * zb + (double)dcorZ);
    return nblk;
}

/* ------------------------------------------------------------------------ */
/* FP32 restatement                                                          */

/* RB_comma3DKernel, kernel.cu:179-201 (in place, layout [H][N][W]). */
void orc_weight_f32(float *sino, const orc_geom *g)
{
    for (int r = 0; r < g->H; ++r) {
        float cs = (float)r - g->cZ;
        for (int b = 0; b < g->N; ++b) {
            float *row = sino + ((size_t)r * g->N + b) * g->W;
            for (int x = 0; x < g->W; ++x) {
                float ce = (float)x - g->cX;
                row[x] *= g->D / sqrtf(ce * ce + g->D * g->D + cs * cs);
            }
        }
    }
}

typedef struct {
    const float *in;
    float *out;
    const orc_geom *g;
    const float *Hf; /* p/2+1 */
    const float *tw; /* p/2 complex */
    int p;
} orc_filt32_ctx;

static void orc_filt32_row(void *vctx, long row)
{
    orc_filt32_ctx *c = (orc_filt32_ctx *)vctx;
    int p = c->p, W = c->g->W;
    float *re = (float *)malloc(sizeof(float) * 2 * (size_t)p);
    float *im = re + p;
    const float *src = c->in + (size_t)row * W;
    for (int i = 0; i < p; ++i) { re[i] = i < W ? src[i] : 0.f; im[i] = 0.f; }
    orc_fft_f32(re, im, p, c->tw, -1);
    for (int k = 0; k < p; ++k) {
        float h = c->Hf[k <= p / 2 ? k : p - k];
        re[k] *= h;
        im[k] *= h;
    }
    orc_fft_f32(re, im, p, c->tw, +1);
    float *dst = c->out + (size_t)row * W;
    for (int i = 0; i < W; ++i) dst[i] = re[i];
    free(re);
}

/* fConvolution, kernel.cu:557-781: per row R2C (zero padded to p), multiply by
 * tau*|FFT(h)|, unnormalised C2R.  Own FP32 FFT stands in for cuFFT. */
void orc_filter_f32(const float *weighted, float *q, const orc_geom *g, int window, int nthreads)
{
    int W = g->W, p = orc_pad_length(W);
    double *tw64 = (double *)malloc(sizeof(double) * (size_t)p);
    orc_twiddles_f64(tw64, p);
    float *tw = (float *)malloc(sizeof(float) * (size_t)p);
    for (int i = 0; i < p; ++i) tw[i] = (float)tw64[i];
    /* filter spectrum exactly as AbsKernel builds it, in FP32 */
    float *re = (float *)calloc(2 * (size_t)p, sizeof(float));
    float *im = re + p;
    for (int i = 0; i < W; ++i) re[i] = orc_ramlak(i - W / 2, g->tau) / 2;
    orc_fft_f32(re, im, p, tw, -1);
    float *Hf = (float *)malloc(sizeof(float) * (size_t)(p / 2 + 1));
    for (int k = 0; k <= p / 2; ++k) {
        float X = re[k], Y = im[k];
        Hf[k] = g->tau * sqrtf(X * X + Y * Y);
        if (window != ORC_WIN_RAMLAK) Hf[k] = (float)(Hf[k] * orc_window(window, k, p));
    }
    orc_filt32_ctx c = {weighted, q, g, Hf, tw, p};
    orc_parallel_for((long)g->H * g->N, nthreads, orc_filt32_row, &c);
    free(tw64); free(tw); free(re); free(Hf);
}

/* fQ3D, kernel.cu:121-177, on one contiguous [H][N][W] sinogram. */
static float orc_fq3d(float p_, float f_, int beta, const float *q, const orc_geom *g)
{
    float scP = p_ + g->cX;
    float scF = f_ + g->cZ;
    if ((scP < 0) || (scP > (float)(g->W - 1))) return 0;
    if ((scF < 0) || (scF > (float)(g->H - 1))) return 0;
    int af = (int)ceilf(scF);
    int bf = (int)floorf(scF);
    int a = (int)ceilf(scP);
    int b = (int)floorf(scP);
    const float *rowa = q + ((size_t)af * g->N + beta) * g->W;
    if (af != bf) {
        const float *rowb = q + ((size_t)bf * g->N + beta) * g->W;
        float va, vb;
        if (a != b) {
            va = (rowa[a] + (rowa[b] - rowa[a]) * (-scP + (float)a));
            vb = (rowb[a] + (rowb[b] - rowb[a]) * (-scP + (float)a));
        } else {
            va = rowa[a];
            vb = rowb[b];
        }
        return (va + (vb - va) * (-scF + (float)af));
    }
    if (a != b) return (rowa[a] + (rowa[b] - rowa[a]) * (-scP + (float)a));
    return rowa[a];
}

/* CalcSinCos, kernel.cu:430-441: the angle is formed in float, then sin/cos
 * in double, stored as float. */
static void orc_sincos_tables(const orc_geom *g, float *sn, float *cs)
{
    for (int b = 0; b < g->N; ++b) {
        float bf = (float)b * g->dfi;
        double beta_rad = (double)(float)(bf + g->rot);
        sn[b] = (float)sin(beta_rad);
        cs[b] = (float)cos(beta_rad);
    }
}

static double orc_angle(const orc_geom *g, int b)
{
    float bf = (float)b * g->dfi;
    return (double)(float)(bf + g->rot);
}

typedef struct {
    const float *q;
    const orc_geom *g;
    const int *zlist;
    float *vol;
    const float *sn, *cs;
    const float *zoff;
    int nblk, zb;
    float dX, dY, fscale;
} orc_bp32_ctx;

static inline float orc_flip(float v, int on) { return on ? -v : v; }

static void orc_bp32_row(void *vctx, long idx)
{
    orc_bp32_ctx *c = (orc_bp32_ctx *)vctx;
    const orc_geom *g = c->g;
    int zi = (int)(idx / g->Y), y = (int)(idx % g->Y);
    int z = c->zlist[zi];
    float *out = c->vol + ((size_t)zi * g->Y + y) * g->X;
    int n = z / c->zb, zl = z - n * c->zb;
    if (n >= c->nblk || z < 0 || z >= g->Z) { /* slice never computed by the reference */
        for (int x = 0; x < g->X; ++x) out[x] = 0.f;
        return;
    }
    float aY = orc_flip(g->scale * ((float)y + c->dY), g->diry);
    float aZ = orc_flip(g->scale * ((float)zl + c->zoff[n]), g->dirz);
    for (int x = 0; x < g->X; ++x) {
        float aX = orc_flip(g->scale * ((float)x + c->dX), g->dirx);
        float result = 0;
        if (sqrtf(aX * aX + aY * aY) < g->W / 2.) {
            for (int b = 0; b < g->N; ++b) {
                float dsin = c->sn[b], dcos = c->cs[b];
                float S = aX * dcos + aY * dsin;
                float T = aY * dcos - aX * dsin;
                float U = g->D / (g->D - S);
                result += U * U * orc_fq3d(T * U, aZ * U, b, c->q, g);
            }
            result *= c->fscale;
        }
        out[x] = result;
    }
}

/* FBPConeKernel, kernel.cu:68-119, over the listed output slices. */
void orc_bp_f32(const float *q, const orc_geom *g, const int *zlist, int nz, float *vol, int nthreads)
{
    float *sn = (float *)malloc(sizeof(float) * (size_t)g->N * 2);
    float *cs = sn + g->N;
    orc_sincos_tables(g, sn, cs);
    float zoff[65536];
    int nblk = orc_zblocks(g, zoff, 65536);
    float scaling = 1.f / (float)orc_pad_length(g->W); /* sing.scaling /= p */
    orc_bp32_ctx c;
    c.q = q; c.g = g; c.zlist = zlist; c.vol = vol; c.sn = sn; c.cs = cs;
    c.zoff = zoff; c.nblk = nblk; c.zb = g->zb > 0 ? g->zb : 16;
    c.dX = -g->cx; c.dY = -g->cy;
    c.fscale = g->dfi * scaling;
    orc_parallel_for((long)nz * g->Y, nthreads, orc_bp32_row, &c);
    free(sn);
}

int orc_fdk_f32(const float *sino, const orc_geom *g, int window,
                const int *zlist, int nz, float *vol, int nthreads)
{
    size_t n = (size_t)g->W * g->N * g->H;
    float *w = (float *)malloc(sizeof(float) * n);
    float *q = (float *)malloc(sizeof(float) * n);
    if (!w || !q) { free(w); free(q); return -1; }
    memcpy(w, sino, sizeof(float) * n);
    orc_weight_f32(w, g);
    orc_filter_f32(w, q, g, window, nthreads);
    orc_bp_f32(q, g, zlist, nz, vol, nthreads);
    free(w); free(q);
    return 0;
}

typedef struct {
    const uint16_t *raw;
    float *band; /* [nrows][N][W] */
    const orc_geom *g;
    int row_lo;
    double dark, flat, A, B, fl;
    int invert;
} orc_prep_ctx;

/* log (rsq_load.cpp:299-325) then cosine weight (kernel.cu:179-201) of one
 * (row, angle) line of the band. */
static void orc_prep_row(void *vctx, long i)
{
    orc_prep_ctx *c = (orc_prep_ctx *)vctx;
    const orc_geom *g = c->g;
    int rr = (int)(i / g->N), b = (int)(i % g->N), r = c->row_lo + rr;
    const uint16_t *src = c->raw + ((size_t)b * g->H + r) * g->W;
    float *dst = c->band + ((size_t)rr * g->N + b) * g->W;
    float cs = (float)r - g->cZ;
    for (int x = 0; x < g->W; ++x) {
        double num = (double)src[x] - c->dark, den = c->flat - c->dark;
        if (num < c->fl) num = c->fl;
        if (den < c->fl) den = c->fl;
        double v = c->A * log(num / den) + c->B;
        float fv = (float)(c->invert ? -v : v);
        float ce = (float)x - g->cX;
        dst[x] = fv * (g->D / sqrtf(ce * ce + g->D * g->D + cs * cs));
    }
}

int orc_fdk_u16_f32_sampled(const uint16_t *raw, double dark, double flat, double A, double B, int invert,
                            double floor_counts, const orc_geom *g, int window,
                            const int *zlist, int nz, float *vol, int nthreads)
{
    int lo, hi;
    orc_rows_needed(g, zlist, nz, &lo, &hi);
    size_t plane = (size_t)g->N * g->W, nr = (size_t)(hi - lo + 1);
    float *band = (float *)malloc(sizeof(float) * nr * plane);
    float *q = (float *)calloc((size_t)g->H * plane, sizeof(float)); /* rows outside the band stay 0 */
    if (!band || !q) { free(band); free(q); return -1; }
    orc_prep_ctx pc = {raw, band, g, lo, dark, flat, A, B, floor_counts, invert};
    orc_parallel_for((long)nr * g->N, nthreads, orc_prep_row, &pc);
    orc_geom gb = *g;
    gb.H = (int)nr;
    orc_filter_f32(band, q + (size_t)lo * plane, &gb, window, nthreads);
    orc_bp_f32(q, g, zlist, nz, vol, nthreads);
    free(band); free(q);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* FP64 oracle                                                               */

void orc_rows_needed(const orc_geom *g, const int *zlist, int nz, int *lo, int *hi)
{
    double D = g->D, R = g->W / 2.0;
    double umin = D / (D + R), umax = R < D ? D / (D - R) : 1e30;
    double vlo = 1e300, vhi = -1e300;
    for (int i = 0; i < nz; ++i) {
        double aZ = g->scale * ((double)zlist[i] - (g->Z - 1) / 2.0 - g->cz);
        if (g->dirz) aZ = -aZ;
        double v1 = aZ * umin + g->cZ, v2 = aZ * umax + g->cZ;
        if (v1 < vlo) vlo = v1;
        if (v2 < vlo) vlo = v2;
        if (v1 > vhi) vhi = v1;
        if (v2 > vhi) vhi = v2;
    }
    int l = (int)floor(vlo) - 1, h = (int)ceil(vhi) + 1;
    if (l < 0) l = 0;
    if (h > g->H - 1) h = g->H - 1;
    if (h < l) h = l;
    *lo = l;
    *hi = h;
}

typedef struct {
    const float *sino;
    double *q;
    const orc_geom *g;
    const double *Hf, *tw;
    int p, row_lo;
} orc_filt64_ctx;

static void orc_filt64_row(void *vctx, long i)
{
    orc_filt64_ctx *c = (orc_filt64_ctx *)vctx;
    const orc_geom *g = c->g;
    int p = c->p, W = g->W;
    int r = c->row_lo + (int)(i / g->N), b = (int)(i % g->N);
    double *re = (double *)malloc(sizeof(double) * 2 * (size_t)p);
    double *im = re + p;
    const float *src = c->sino + ((size_t)r * g->N + b) * W;
    double D = g->D, cs = (double)r - g->cZ;
    for (int x = 0; x < p; ++x) {
        im[x] = 0;
        if (x < W) {
            double ce = (double)x - g->cX;
            re[x] = (double)src[x] * D / sqrt(ce * ce + D * D + cs * cs);
        } else {
            re[x] = 0;
        }
    }
    orc_fft_f64(re, im, p, c->tw, -1);
    for (int k = 0; k < p; ++k) {
        double h = c->Hf[k <= p / 2 ? k : p - k];
        re[k] *= h;
        im[k] *= h;
    }
    orc_fft_f64(re, im, p, c->tw, +1);
    double *dst = c->q + (size_t)i * W;
    for (int x = 0; x < W; ++x) dst[x] = re[x] / (double)p;
    free(re);
}

/* Cosine weight + ramp filter in double for detector rows [row_lo, row_hi];
 * q64 is [row_hi-row_lo+1][N][W]. */
void orc_weight_filter_f64(const float *sino, double *q64, const orc_geom *g, int window,
                           int row_lo, int row_hi, int nthreads)
{
    int p = orc_pad_length(g->W);
    double *Hf = (double *)malloc(sizeof(double) * (size_t)(p / 2 + 1));
    orc_spectrum_f64(g->W, g->tau, window, p, Hf);
    double *tw = (double *)malloc(sizeof(double) * (size_t)p);
    orc_twiddles_f64(tw, p);
    orc_filt64_ctx c = {sino, q64, g, Hf, tw, p, row_lo};
    orc_parallel_for((long)(row_hi - row_lo + 1) * g->N, nthreads, orc_filt64_row, &c);
    free(Hf); free(tw);
}

typedef struct {
    const double *q;
    const orc_geom *g;
    const int *zlist;
    double *vol;
    const double *sn, *cs;
    int row_lo, nrows;
} orc_bp64_ctx;

static double orc_fq64(double u, double v, int beta, const orc_bp64_ctx *c)
{
    const orc_geom *g = c->g;
    if (u < 0 || u > g->W - 1 || v < 0 || v > g->H - 1) return 0;
    int a = (int)floor(u), b = (int)floor(v);
    double fu = u - a, fv = v - b;
    int a1 = a + 1 < g->W ? a + 1 : a, b1 = b + 1 < g->H ? b + 1 : b;
    int rb = b - c->row_lo, rb1 = b1 - c->row_lo;
    if (rb < 0 || rb1 >= c->nrows) return NAN; /* row band too small: make it loud */
    const double *r0 = c->q + ((size_t)rb * g->N + beta) * g->W;
    const double *r1 = c->q + ((size_t)rb1 * g->N + beta) * g->W;
    double top = r0[a] + (r0[a1] - r0[a]) * fu;
    double bot = r1[a] + (r1[a1] - r1[a]) * fu;
    return top + (bot - top) * fv;
}

static void orc_bp64_row(void *vctx, long idx)
{
    orc_bp64_ctx *c = (orc_bp64_ctx *)vctx;
    const orc_geom *g = c->g;
    int zi = (int)(idx / g->Y), y = (int)(idx % g->Y);
    int z = c->zlist[zi];
    double *out = c->vol + ((size_t)zi * g->Y + y) * g->X;
    double s = g->scale, D = g->D;
    double aY = s * ((double)y - g->cy);
    double aZ = s * ((double)z - (g->Z - 1) / 2.0 - g->cz);
    if (g->diry) aY = -aY;
    if (g->dirz) aZ = -aZ;
    for (int x = 0; x < g->X; ++x) {
        double aX = s * ((double)x - g->cx);
        if (g->dirx) aX = -aX;
        double result = 0;
        if (sqrt(aX * aX + aY * aY) < g->W / 2.0) {
            for (int b = 0; b < g->N; ++b) {
                double S = aX * c->cs[b] + aY * c->sn[b];
                double T = aY * c->cs[b] - aX * c->sn[b];
                double U = D / (D - S);
                result += U * U * orc_fq64(T * U + g->cX, aZ * U + g->cZ, b, c);
            }
            result *= (double)g->dfi;
        }
        out[x] = result;
    }
}

void orc_bp_f64(const double *q64, const orc_geom *g, const int *zlist, int nz, double *vol,
                int row_lo, int nthreads)
{
    int lo, hi;
    orc_rows_needed(g, zlist, nz, &lo, &hi);
    double *sn = (double *)malloc(sizeof(double) * 2 * (size_t)g->N);
    double *cs = sn + g->N;
    for (int b = 0; b < g->N; ++b) {
        double a = orc_angle(g, b);
        sn[b] = sin(a);
        cs[b] = cos(a);
    }
    orc_bp64_ctx c;
    c.q = q64; c.g = g; c.zlist = zlist; c.vol = vol; c.sn = sn; c.cs = cs;
    c.row_lo = row_lo;
    c.nrows = hi - row_lo + 1;
    if (c.nrows < 1) c.nrows = 1;
    orc_parallel_for((long)nz * g->Y, nthreads, orc_bp64_row, &c);
    free(sn);
}

int orc_fdk_f64(const float *sino, const orc_geom *g, int window,
                const int *zlist, int nz, double *vol, int nthreads)
{
    int lo, hi;
    orc_rows_needed(g, zlist, nz, &lo, &hi);
    size_t n = (size_t)(hi - lo + 1) * g->N * g->W;
    double *q = (double *)malloc(sizeof(double) * n);
    if (!q) return -1;
    orc_weight_filter_f64(sino, q, g, window, lo, hi, nthreads);
    orc_bp_f64(q, g, zlist, nz, vol, lo, nthreads);
    free(q);
    return 0;
}

/* FP64 FDK of raw uint16 counts on listed slices, with the projections taken
 * in blocks of ORC_U16_BLOCK so that memory stays O(rows x block x W) however
 * many projections there are: log as orc_log_u16_f64 with scalar dark/flat
 * (rsq_load.cpp:299-325) kept in double, cosine weight (kernel.cu:179-201),
 * ramp filter (kernel.cu:557-802) and bilinear backprojection
 * (kernel.cu:68-177), all in double. */
#define ORC_U16_BLOCK 16

typedef struct {
    const uint16_t *raw;
    const orc_geom *g;
    double *q; /* [nr][nb][W] */
    const double *Hf, *tw;
    int p, row_lo, b0, nb;
    double dark, flat, A, B, fl;
    int invert;
} orc_u16f64_filt_ctx;

static void orc_u16f64_filt_row(void *vctx, long i)
{
    orc_u16f64_filt_ctx *c = (orc_u16f64_filt_ctx *)vctx;
    const orc_geom *g = c->g;
    int p = c->p, W = g->W;
    int rr = (int)(i / c->nb), bb = (int)(i % c->nb), r = c->row_lo + rr, b = c->b0 + bb;
    double *re = (double *)malloc(sizeof(double) * 2 * (size_t)p);
    double *im = re + p;
    const uint16_t *src = c->raw + ((size_t)b * g->H + r) * W;
    double D = g->D, cs = (double)r - g->cZ;
    double den = c->flat - c->dark;
    if (den < c->fl) den = c->fl;
    for (int x = 0; x < p; ++x) {
        im[x] = 0;
        re[x] = 0;
        if (x < W) {
            double num = (double)src[x] - c->dark;
            if (num < c->fl) num = c->fl;
            double v = c->A * log(num / den) + c->B;
            if (c->invert) v = -v;
            double ce = (double)x - g->cX;
            re[x] = v * D / sqrt(ce * ce + D * D + cs * cs);
        }
    }
    orc_fft_f64(re, im, p, c->tw, -1);
    for (int k = 0; k < p; ++k) {
        double h = c->Hf[k <= p / 2 ? k : p - k];
        re[k] *= h;
        im[k] *= h;
    }
    orc_fft_f64(re, im, p, c->tw, +1);
    double *dst = c->q + ((size_t)rr * c->nb + bb) * W;
    for (int x = 0; x < W; ++x) dst[x] = re[x] / (double)p;
    free(re);
}

typedef struct {
    const double *q;
    const orc_geom *g;
    const int *zlist;
    double *vol;
    const double *sn, *cs;
    int row_lo, nrows, b0, nb;
} orc_u16f64_bp_ctx;

static void orc_u16f64_bp_row(void *vctx, long idx)
{
    orc_u16f64_bp_ctx *c = (orc_u16f64_bp_ctx *)vctx;
    const orc_geom *g = c->g;
    int zi = (int)(idx / g->Y), y = (int)(idx % g->Y);
    double *out = c->vol + ((size_t)zi * g->Y + y) * g->X;
    double s = g->scale, D = g->D;
    double aY = s * ((double)y - g->cy);
    double aZ = s * ((double)c->zlist[zi] - (g->Z - 1) / 2.0 - g->cz);
    if (g->diry) aY = -aY;
    if (g->dirz) aZ = -aZ;
    for (int x = 0; x < g->X; ++x) {
        double aX = s * ((double)x - g->cx);
        if (g->dirx) aX = -aX;
        if (!(sqrt(aX * aX + aY * aY) < g->W / 2.0)) continue;
        double acc = 0;
        for (int bb = 0; bb < c->nb; ++bb) {
            int b = c->b0 + bb;
            double S = aX * c->cs[b] + aY * c->sn[b];
            double T = aY * c->cs[b] - aX * c->sn[b];
            double U = D / (D - S);
            double u = T * U + g->cX, v = aZ * U + g->cZ;
            if (u < 0 || u > g->W - 1 || v < 0 || v > g->H - 1) continue;
            int a = (int)floor(u), r = (int)floor(v);
            double fu = u - a, fv = v - r;
            int a1 = a + 1 < g->W ? a + 1 : a, r1 = r + 1 < g->H ? r + 1 : r;
            int rb = r - c->row_lo, rb1 = r1 - c->row_lo;
            if (rb < 0 || rb1 >= c->nrows) { acc = NAN; break; } /* band too small: make it loud */
            const double *q0 = c->q + ((size_t)rb * c->nb + bb) * g->W;
            const double *q1 = c->q + ((size_t)rb1 * c->nb + bb) * g->W;
            double top = q0[a] + (q0[a1] - q0[a]) * fu;
            double bot = q1[a] + (q1[a1] - q1[a]) * fu;
            acc += U * U * (top + (bot - top) * fv);
        }
        out[x] += acc;
    }
}

int orc_fdk_u16_f64_sampled(const uint16_t *raw, double dark, double flat, double A, double B, int invert,
                            double floor_counts, const orc_geom *g, int window,
                            const int *zlist, int nz, double *vol, int nthreads)
{
    int lo, hi;
    orc_rows_needed(g, zlist, nz, &lo, &hi);
    int nr = hi - lo + 1, nb = g->N < ORC_U16_BLOCK ? g->N : ORC_U16_BLOCK;
    int p = orc_pad_length(g->W);
    double *q = (double *)malloc(sizeof(double) * (size_t)nr * nb * g->W);
    double *Hf = (double *)malloc(sizeof(double) * (size_t)(p / 2 + 1));
    double *tw = (double *)malloc(sizeof(double) * (size_t)p);
    double *sn = (double *)malloc(sizeof(double) * 2 * (size_t)g->N);
    if (!q || !Hf || !tw || !sn) { free(q); free(Hf); free(tw); free(sn); return -1; }
    double *cs = sn + g->N;
    orc_spectrum_f64(g->W, g->tau, window, p, Hf);
    orc_twiddles_f64(tw, p);
    for (int b = 0; b < g->N; ++b) {
        double a = orc_angle(g, b);
        sn[b] = sin(a);
        cs[b] = cos(a);
    }
    size_t nvox = (size_t)nz * g->Y * g->X;
    memset(vol, 0, sizeof(double) * nvox);
    for (int b0 = 0; b0 < g->N; b0 += nb) {
        int nbb = g->N - b0 < nb ? g->N - b0 : nb;
        orc_u16f64_filt_ctx fc = {raw, g, q, Hf, tw, p, lo, b0, nbb, dark, flat, A, B, floor_counts, invert};
        orc_parallel_for((long)nr * nbb, nthreads, orc_u16f64_filt_row, &fc);
        orc_u16f64_bp_ctx bc = {q, g, zlist, vol, sn, cs, lo, nr, b0, nbb};
        orc_parallel_for((long)nz * g->Y, nthreads, orc_u16f64_bp_row, &bc);
    }
    for (size_t i = 0; i < nvox; ++i) vol[i] *= (double)g->dfi;
    free(q); free(Hf); free(tw); free(sn);
    return 0;
}

/* Half-fan completion and fan->parallel rebinning in double, restating
 * rsq::Half2FullFan (rsq_load.cpp:327-380) and rsq::Half2Para/Fan2Para
 * (rsq_load.cpp:382-470) for `rows` independent [N][W] sinograms.  Angle
 * indices past the last angle wrap to the first as in the reference. */
static int orc_wrap(int a, int N)
{
    if (a > N - 1) a -= N;
    if (a < 0) a += N;
    return a;
}

void orc_half2fullfan_f64(const double *in, int W, int N, int rows, int am, double D, double dfi, int flip,
                          double *out)
{
    int Wc = 2 * W - 1 - 2 * am, c0 = W - 1 - am;
    for (int r = 0; r < rows; ++r) {
        const double *img = in + (size_t)r * N * W;
        for (int f = 0; f < N; ++f) {
            double *row = out + ((size_t)r * N + (flip ? N - 1 - f : f)) * Wc;
            for (int c = c0; c < Wc; ++c) row[c] = img[(size_t)f * W + (c - c0) + am];
            double fi = f * dfi;
            for (int t = -c0; t < 0; ++t) {
                double at = atan(t / D);
                double nf = (fi - 2 * at - ORC_PI) / dfi;
                if (nf > (N - 1) || nf < 0) nf = (fi - 2 * at + ORC_PI) / dfi;
                int a = (int)ceil(nf), b = (int)floor(nf);
                double A = img[(size_t)orc_wrap(a, N) * W + (-t) + am];
                double B = img[(size_t)orc_wrap(b, N) * W + (-t) + am];
                row[t + c0] = (a != b) ? A + (B - A) * (-nf + a) : A;
            }
        }
    }
}

void orc_half2para_f64(const double *in, int W, int N, int rows, int am, double D, double dfi, double *out)
{
    int Wc = 2 * W - 1 - 2 * am, Np = N / 2, center = W - 1 - am;
    for (int r = 0; r < rows; ++r) {
        const double *img = in + (size_t)r * N * W;
        for (int f = 0; f < Np; ++f)
            for (int u = 0; u < Wc; ++u) {
                double ui = (double)u - (double)center, beta, s = ui;
                if (ui >= 0.) beta = f + asin(ui / D) / dfi;
                else beta = f - (asin(ui / D) - ORC_PI) / dfi;
                if (beta < 0.) beta += N;
                if (beta > N - 1) beta -= N;
                if (ui < 0.) s *= -1;
                int ba = (int)ceil(beta), bb = (int)floor(beta);
                int sa = (int)ceil(s);
                int col = sa + am; /* both taps use the ceiling (rsq_load.cpp:436-437) */
                double v;
                if (ba != bb) {
                    double va = img[(size_t)orc_wrap(ba, N) * W + col];
                    double vb = img[(size_t)orc_wrap(bb, N) * W + col];
                    v = va + (vb - va) * (-beta + ba);
                } else {
                    v = img[(size_t)orc_wrap(ba, N) * W + col];
                }
                out[((size_t)r * Np + f) * Wc + u] = v;
            }
    }
}

/* adjoint: scatter every voxel into the filtered-sample gradient, one
 * projection per task (no races), then filter and weight each row */
typedef struct {
    const float *vol;
    const orc_geom *g;
    double *qbar; /* [N][H][W] */
    const double *sn, *cs;
} orc_adj_ctx;

static void orc_adj_proj(void *vctx, long b)
{
    orc_adj_ctx *c = (orc_adj_ctx *)vctx;
    const orc_geom *g = c->g;
    double *q = c->qbar + (size_t)b * g->H * g->W;
    double s = g->scale, D = g->D;
    for (int z = 0; z < g->Z; ++z) {
        double aZ = s * ((double)z - (g->Z - 1) / 2.0 - g->cz);
        if (g->dirz) aZ = -aZ;
        for (int y = 0; y < g->Y; ++y) {
            double aY = s * ((double)y - g->cy);
            if (g->diry) aY = -aY;
            for (int x = 0; x < g->X; ++x) {
                double aX = s * ((double)x - g->cx);
                if (g->dirx) aX = -aX;
                if (!(sqrt(aX * aX + aY * aY) < g->W / 2.0)) continue;
                double val = c->vol[((size_t)z * g->Y + y) * g->X + x];
                if (val == 0) continue;
                double S = aX * c->cs[b] + aY * c->sn[b];
                double T = aY * c->cs[b] - aX * c->sn[b];
                double U = D / (D - S);
                double u = T * U + g->cX, v = aZ * U + g->cZ;
                if (u < 0 || u > g->W - 1 || v < 0 || v > g->H - 1) continue;
                int a = (int)floor(u), r = (int)floor(v);
                double fu = u - a, fv = v - r;
                double w = (double)g->dfi * U * U * val;
                int a1 = a + 1 < g->W ? a + 1 : a, r1 = r + 1 < g->H ? r + 1 : r;
                q[(size_t)r * g->W + a] += w * (1 - fu) * (1 - fv);
                q[(size_t)r * g->W + a1] += w * fu * (1 - fv);
                q[(size_t)r1 * g->W + a] += w * (1 - fu) * fv;
                q[(size_t)r1 * g->W + a1] += w * fu * fv;
            }
        }
    }
}

typedef struct {
    const double *qbar;
    double *out;
    const orc_geom *g;
    const double *Hf, *tw;
    int p;
} orc_adjf_ctx;

static void orc_adj_filter_row(void *vctx, long i)
{
    orc_adjf_ctx *c = (orc_adjf_ctx *)vctx;
    const orc_geom *g = c->g;
    int p = c->p, W = g->W;
    int b = (int)(i / g->H), r = (int)(i % g->H);
    double *re = (double *)malloc(sizeof(double) * 2 * (size_t)p);
    double *im = re + p;
    const double *src = c->qbar + (size_t)i * W;
    for (int x = 0; x < p; ++x) { re[x] = x < W ? src[x] : 0; im[x] = 0; }
    orc_fft_f64(re, im, p, c->tw, -1);
    for (int k = 0; k < p; ++k) {
        double h = c->Hf[k <= p / 2 ? k : p - k];
        re[k] *= h;
        im[k] *= h;
    }
    orc_fft_f64(re, im, p, c->tw, +1);
    double D = g->D, cs = (double)r - g->cZ;
    double *dst = c->out + ((size_t)r * g->N + b) * W;
    for (int x = 0; x < W; ++x) {
        double ce = (double)x - g->cX;
        dst[x] = re[x] / (double)p * (D / sqrt(ce * ce + D * D + cs * cs));
    }
    free(re);
}

int orc_fdk_adjoint_f64(const float *vol, const orc_geom *g, int window, double *out, int nthreads)
{
    size_t nq = (size_t)g->N * g->H * g->W;
    double *qbar = (double *)calloc(nq, sizeof(double));
    double *sn = (double *)malloc(sizeof(double) * 2 * (size_t)g->N);
    if (!qbar || !sn) { free(qbar); free(sn); return -1; }
    double *cs = sn + g->N;
    for (int b = 0; b < g->N; ++b) {
        double a = orc_angle(g, b);
        sn[b] = sin(a);
        cs[b] = cos(a);
    }
    orc_adj_ctx c = {vol, g, qbar, sn, cs};
    orc_parallel_for(g->N, nthreads, orc_adj_proj, &c);
    int p = orc_pad_length(g->W);
    double *Hf = (double *)malloc(sizeof(double) * (size_t)(p / 2 + 1));
    double *tw = (double *)malloc(sizeof(double) * (size_t)p);
    orc_spectrum_f64(g->W, g->tau, window, p, Hf);
    orc_twiddles_f64(tw, p);
    orc_adjf_ctx f = {qbar, out, g, Hf, tw, p};
    orc_parallel_for((long)g->N * g->H, nthreads, orc_adj_filter_row, &f);
    free(qbar); free(sn); free(Hf); free(tw);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* The plain backprojection pair of the volume data-consistency refinement
 * (tk_refine_volume), in double:
 *   B:   vol[z][y][x] = (dfi/p) sum_b U^2 Q_b(u, v), the bilinear backprojection
 *        of FBPConeKernel + fQ3D (kernel.cu:68-177) with the reference's final
 *        scale delta_f * (1/p) (kernel.cu:113, 575), zero outside the detector
 *        and outside the FOV cylinder;
 *   B^T: its exact transpose, q[b][r][c] += (dfi/p) U^2 w_rc vol for the four
 *        bilinear weights w_rc of every voxel.
 * q is [N][H][W]; slice z sits at aZ = s (z - (Z-1)/2 - cz). */
typedef struct {
    const orc_geom *g;
    const double *sn, *cs;
    double fs;
    const double *vin;
    double *qout;
    const double *qin;
    double *vout;
} orc_pair_ctx;

static int orc_pair_coords(const orc_geom *g, int x, int y, int z, double *aX, double *aY, double *aZ)
{
    double s = g->scale;
    *aX = s * ((double)x - g->cx);
    *aY = s * ((double)y - g->cy);
    *aZ = s * ((double)z - (g->Z - 1) / 2.0 - g->cz);
    if (g->dirx) *aX = -*aX;
    if (g->diry) *aY = -*aY;
    if (g->dirz) *aZ = -*aZ;
    return sqrt(*aX * *aX + *aY * *aY) < g->W / 2.0;
}

static void orc_bt_proj(void *vctx, long b)
{
    orc_pair_ctx *c = (orc_pair_ctx *)vctx;
    const orc_geom *g = c->g;
    double *q = c->qout + (size_t)b * g->H * g->W;
    for (int z = 0; z < g->Z; ++z)
        for (int y = 0; y < g->Y; ++y)
            for (int x = 0; x < g->X; ++x) {
                double aX, aY, aZ;
                if (!orc_pair_coords(g, x, y, z, &aX, &aY, &aZ)) continue;
                double val = c->vin[((size_t)z * g->Y + y) * g->X + x];
                if (val == 0) continue;
                double S = aX * c->cs[b] + aY * c->sn[b], T = aY * c->cs[b] - aX * c->sn[b];
                double U = g->D / (g->D - S), u = T * U + g->cX, v = aZ * U + g->cZ;
                if (u < 0 || u > g->W - 1 || v < 0 || v > g->H - 1) continue;
                int a = (int)floor(u), r = (int)floor(v);
                double fu = u - a, fv = v - r, w = c->fs * U * U * val;
                q[(size_t)r * g->W + a] += w * (1 - fu) * (1 - fv);
                if (a + 1 < g->W) q[(size_t)r * g->W + a + 1] += w * fu * (1 - fv);
                if (r + 1 < g->H) {
                    q[(size_t)(r + 1) * g->W + a] += w * (1 - fu) * fv;
                    if (a + 1 < g->W) q[(size_t)(r + 1) * g->W + a + 1] += w * fu * fv;
                }
            }
}

static double orc_q_at(const orc_geom *g, const double *qb, int r, int c)
{
    return (r < g->H && c < g->W) ? qb[(size_t)r * g->W + c] : 0.0;
}

static void orc_b_row(void *vctx, long idx)
{
    orc_pair_ctx *c = (orc_pair_ctx *)vctx;
    const orc_geom *g = c->g;
    int z = (int)(idx / g->Y), y = (int)(idx % g->Y);
    double *out = c->vout + ((size_t)z * g->Y + y) * g->X;
    for (int x = 0; x < g->X; ++x) {
        double aX, aY, aZ, acc = 0;
        if (orc_pair_coords(g, x, y, z, &aX, &aY, &aZ)) {
            for (int b = 0; b < g->N; ++b) {
                double S = aX * c->cs[b] + aY * c->sn[b], T = aY * c->cs[b] - aX * c->sn[b];
                double U = g->D / (g->D - S), u = T * U + g->cX, v = aZ * U + g->cZ;
                if (u < 0 || u > g->W - 1 || v < 0 || v > g->H - 1) continue;
                int a = (int)floor(u), r = (int)floor(v);
                double fu = u - a, fv = v - r;
                const double *qb = c->qin + (size_t)b * g->H * g->W;
                double top = orc_q_at(g, qb, r, a) * (1 - fu) + orc_q_at(g, qb, r, a + 1) * fu;
                double bot = orc_q_at(g, qb, r + 1, a) * (1 - fu) + orc_q_at(g, qb, r + 1, a + 1) * fu;
                acc += U * U * (top * (1 - fv) + bot * fv);
            }
        }
        out[x] = c->fs * acc;
    }
}

static void orc_pair_setup(const orc_geom *g, orc_pair_ctx *c, double *trig)
{
    c->g = g;
    c->sn = trig;
    c->cs = trig + g->N;
    for (int b = 0; b < g->N; ++b) {
        double a = orc_angle(g, b);
        trig[b] = sin(a);
        trig[g->N + b] = cos(a);
    }
    c->fs = (double)g->dfi / (double)orc_pad_length(g->W);
}

int orc_bt_f64(const double *vol, const orc_geom *g, double *q, int nthreads)
{
    double *trig = (double *)malloc(sizeof(double) * 2 * (size_t)g->N);
    if (!trig) return -1;
    orc_pair_ctx c;
    memset(&c, 0, sizeof(c));
    orc_pair_setup(g, &c, trig);
    memset(q, 0, sizeof(double) * (size_t)g->N * g->H * g->W);
    c.vin = vol;
    c.qout = q;
    orc_parallel_for(g->N, nthreads, orc_bt_proj, &c);
    free(trig);
    return 0;
}

int orc_b_f64(const double *q, const orc_geom *g, double *vol, int nthreads)
{
    double *trig = (double *)malloc(sizeof(double) * 2 * (size_t)g->N);
    if (!trig) return -1;
    orc_pair_ctx c;
    memset(&c, 0, sizeof(c));
    orc_pair_setup(g, &c, trig);
    c.qin = q;
    c.vout = vol;
    orc_parallel_for((long)g->Z * g->Y, nthreads, orc_b_row, &c);
    free(trig);
    return 0;
}

/* ------------------------------------------------------------------------ */
/* raw uint16 -> line integral (rsq::FlatFieldCorrection, rsq_load.cpp:299-325) */

typedef struct {
    const uint16_t *raw;
    const float *dark, *flat;
    int W, N, H, invert;
    double A, B, fl;
    float *out;
} orc_log_ctx;

static void orc_log_row(void *vctx, long i)
{
    orc_log_ctx *c = (orc_log_ctx *)vctx;
    int b = (int)(i / c->H), r = (int)(i % c->H);
    const uint16_t *src = c->raw + ((size_t)b * c->H + r) * c->W;
    float *dst = c->out + ((size_t)r * c->N + b) * c->W;
    for (int x = 0; x < c->W; ++x) {
        double dk = c->dark ? c->dark[(size_t)r * c->W + x] : 0.0;
        double fl = c->flat[(size_t)r * c->W + x];
        double num = (double)src[x] - dk, den = fl - dk;
        if (num < c->fl) num = c->fl;
        if (den < c->fl) den = c->fl;
        double v = c->A * log(num / den) + c->B;
        dst[x] = (float)(c->invert ? -v : v);
    }
}

void orc_log_u16_f64(const uint16_t *raw, const float *dark, const float *flat,
                     int W, int N, int H, double A, double B, int invert,
                     double floor_counts, float *out_sino, int nthreads)
{
    orc_log_ctx c = {raw, dark, flat, W, N, H, invert, A, B, floor_counts, out_sino};
    orc_parallel_for((long)N * H, nthreads, orc_log_row, &c);
}

/* ------------------------------------------------------------------------ */
/* analytic phantom                                                          */

typedef struct {
    const double *ell;
    int nell;
    const orc_geom *g;
    int layout;
    float *out;
} orc_proj_ctx;

/* Chord length (cm) of the line P(t) = s + t d through ellipsoid e. */
static double orc_chord(const double *e, const double s[3], const double d[3])
{
    double A[3], Bv[3];
    for (int i = 0; i < 3; ++i) {
        const double *R = e + 6 + 3 * i;
        double ad = R[0] * d[0] + R[1] * d[1] + R[2] * d[2];
        double as = R[0] * (s[0] - e[0]) + R[1] * (s[1] - e[1]) + R[2] * (s[2] - e[2]);
        A[i] = ad / e[3 + i];
        Bv[i] = as / e[3 + i];
    }
    double a2 = A[0] * A[0] + A[1] * A[1] + A[2] * A[2];
    double bb = A[0] * Bv[0] + A[1] * Bv[1] + A[2] * Bv[2];
    double c2 = Bv[0] * Bv[0] + Bv[1] * Bv[1] + Bv[2] * Bv[2] - 1.0;
    double disc = bb * bb - a2 * c2;
    if (disc <= 0 || a2 <= 0) return 0;
    double dl = sqrt(d[0] * d[0] + d[1] * d[1] + d[2] * d[2]);
    return 2.0 * sqrt(disc) / a2 * dl;
}

static void orc_proj_row(void *vctx, long i)
{
    orc_proj_ctx *c = (orc_proj_ctx *)vctx;
    const orc_geom *g = c->g;
    int b = (int)(i / g->H), r = (int)(i % g->H);
    double beta = orc_angle(g, b), cb = cos(beta), sb = sin(beta);
    double tau = g->tau, D = g->D;
    double src[3] = {D * cb * tau, D * sb * tau, 0.0};
    double Zd = ((double)r - g->cZ) * tau;
    float *dst = c->layout == 0 ? c->out + ((size_t)r * g->N + b) * g->W
                                : c->out + ((size_t)b * g->H + r) * g->W;
    for (int u = 0; u < g->W; ++u) {
        double T = ((double)u - g->cX) * tau;
        double det[3] = {-T * sb, T * cb, Zd};
        double d[3] = {det[0] - src[0], det[1] - src[1], det[2] - src[2]};
        double acc = 0;
        for (int k = 0; k < c->nell; ++k) {
            const double *e = c->ell + 16 * (size_t)k;
            acc += e[15] * orc_chord(e, src, d);
        }
        dst[u] = (float)acc;
    }
}

void orc_project_ellipsoids(const double *ell, int nell, const orc_geom *g, int layout,
                            float *out, int nthreads)
{
    orc_proj_ctx c = {ell, nell, g, layout, out};
    orc_parallel_for((long)g->N * g->H, nthreads, orc_proj_row, &c);
}

typedef struct {
    const double *ell;
    int nell;
    const orc_geom *g;
    const int *zlist;
    float *vol;
} orc_vox_ctx;

static void orc_vox_row(void *vctx, long idx)
{
    orc_vox_ctx *c = (orc_vox_ctx *)vctx;
    const orc_geom *g = c->g;
    int zi = (int)(idx / g->Y), y = (int)(idx % g->Y);
    double s = g->scale * g->tau;
    double py = s * ((double)y - g->cy);
    double pz = s * ((double)c->zlist[zi] - (g->Z - 1) / 2.0 - g->cz);
    if (g->diry) py = -py;
    if (g->dirz) pz = -pz;
    float *out = c->vol + ((size_t)zi * g->Y + y) * g->X;
    for (int x = 0; x < g->X; ++x) {
        double px = s * ((double)x - g->cx);
        if (g->dirx) px = -px;
        double p[3] = {px, py, pz}, acc = 0;
        for (int k = 0; k < c->nell; ++k) {
            const double *e = c->ell + 16 * (size_t)k;
            double r2 = 0;
            for (int i = 0; i < 3; ++i) {
                const double *R = e + 6 + 3 * i;
                double l = (R[0] * (p[0] - e[0]) + R[1] * (p[1] - e[1]) + R[2] * (p[2] - e[2])) / e[3 + i];
                r2 += l * l;
            }
            if (r2 <= 1.0) acc += e[15];
        }
        out[x] = (float)acc;
    }
}

void orc_voxelise_ellipsoids(const double *ell, int nell, const orc_geom *g,
                             const int *zlist, int nz, float *vol, int nthreads)
{
    orc_vox_ctx c = {ell, nell, g, zlist, vol};
    orc_parallel_for((long)nz * g->Y, nthreads, orc_vox_row, &c);
}
