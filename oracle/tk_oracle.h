/*
 * tk_oracle.h -- CPU oracle for the FDK cone-beam hot path.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the shipped library links, loads or
 * calls this code.  It is used by tests/, by __graft_entry__.smoke() as the
 * checker, and by bench.py's CPU-baseline leg.
 *
 * Two restatements of the reference FDK (Lukas-kV/TomoKvas, FBPG/kernel.cu):
 *   - *_f32: FP32, following the reference's operation order
 *            (cosine weight kernel.cu:179-201, filter kernel.cu:557-802,
 *             backprojection kernel.cu:68-177).
 *   - *_f64: the same discretisation in double precision (the FP64 oracle).
 *
 * Pinned against the reference itself: tests/golden/ref_*.npz hold outputs of
 * the reference's own FBPG/kernel.cu kernels with cuFFT on a GB300
 * (oracle/ref_build.py, oracle/tk_refrun.cpp, tests/golden/make_golden.py);
 * tests/test_golden_reference.py checks both restatements against them, and
 * tests/test_oracle.py adds closed-form consequences of the reference's code.
 *
 * Sinogram layout is the reference's sinogram-major [H][N][W]
 * (detector row, angle, column), FBPG/mucat_file.cpp:244-249.
 * Volume layout is [z][y][x] float, FBPG/kernel.cu:116-117.
 */
#ifndef TK_ORACLE_H
#define TK_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

/* Windows applied to the reference Ram-Lak spectrum. */
enum { ORC_WIN_RAMLAK = 0, ORC_WIN_SHEPP_LOGAN = 1, ORC_WIN_HANN = 2 };

typedef struct orc_geom {
    /* projections: FilteredBackProjection::SetSinogramProperties, kernel.cu:479-497 */
    int W;        /* sin_X: detector columns */
    int N;        /* sin_Y: projections (angles) */
    int H;        /* sin_Z: detector rows */
    float cX;     /* centre of rotation, columns */
    float cZ;     /* vertical detector centre, rows */
    float dfi;    /* angular step, rad */
    float D;      /* source-axis distance in virtual pixels */
    float tau;    /* virtual pixel pitch, cm */
    /* volume: SetReconstructionProperties, kernel.cu:524-537 */
    int X, Y, Z;
    float cx, cy, cz; /* centres passed by the caller (para_TC.cpp:141) */
    float rot;        /* rotation offset, rad */
    float scale;      /* SetScaleXYZ */
    int dirx, diry, dirz; /* SetAxisDirection */
    int zb;           /* SetBlockSize (slices per Z block), reference default 16 */
} orc_geom;

int orc_version(void);

/* Pad length p = 2 * nextpow2(W) starting at 2 (kernel.cu:570-573). */
int orc_pad_length(int W);

/* Effective spatial filter of the reference's FFT filter, normalised so that
 * filtered[i] = sum_j k[i-j] * g[j]; written to k_out[n + W - 1] for
 * n in [-(W-1), W-1].  p <= 0 selects the reference pad length.
 * Returns the pad length used, or -1 on bad arguments. */
int orc_filter_kernel_f64(int W, double tau, int window, int p, double *k_out);

/* Number of Z blocks and the per-block z offset the reference uses
 * (kernel.cu:398-400, 821).  zoff_out[n] receives recn.dZ for block n
 * (capacity >= returned count).  Returns nr_of_Z_blocks. */
int orc_zblocks(const orc_geom *g, float *zoff_out, int cap);

/* FP32 restatement, stage by stage.  q is the reference-scaled filtered
 * sinogram (the output of the reference's C2R before the 1/p applied in
 * the backprojection). */
void orc_weight_f32(float *sino, const orc_geom *g);
void orc_filter_f32(const float *weighted, float *q, const orc_geom *g, int window, int nthreads);
void orc_bp_f32(const float *q, const orc_geom *g, const int *zlist, int nz, float *vol, int nthreads);
/* weight + filter + backprojection; sino is not modified. */
int orc_fdk_f32(const float *sino, const orc_geom *g, int window,
                const int *zlist, int nz, float *vol, int nthreads);

/* FP32 restatement on sampled output slices, from raw uint16 projections
 * [N][H][W] (flat-field + log as orc_log_u16_f64 with scalar dark/flat, then
 * cosine weight, FFT filter, backprojection).  Only the detector rows the
 * slices touch are preprocessed and filtered.  Used as the timed CPU
 * baseline. */
int orc_fdk_u16_f32_sampled(const uint16_t *raw, double dark, double flat, double A, double B, int invert,
                            double floor_counts, const orc_geom *g, int window,
                            const int *zlist, int nz, float *vol, int nthreads);

/* FP64 oracle.  q64 is normalised (no factor p). */
void orc_weight_filter_f64(const float *sino, double *q64, const orc_geom *g, int window,
                           int row_lo, int row_hi, int nthreads);
void orc_bp_f64(const double *q64, const orc_geom *g, const int *zlist, int nz, double *vol,
                int row_lo, int nthreads);
int orc_fdk_f64(const float *sino, const orc_geom *g, int window,
                const int *zlist, int nz, double *vol, int nthreads);
/* FP64 FDK of raw uint16 counts [N][H][W] on listed slices (log, weight,
 * filter and backprojection in double, scalar dark/flat as
 * orc_fdk_u16_f32_sampled), streaming the projections in small blocks so
 * that memory stays O(rows x block x W): the oracle of the out-of-core path.
 * vol [nz][Y][X] double. */
int orc_fdk_u16_f64_sampled(const uint16_t *raw, double dark, double flat, double A, double B, int invert,
                            double floor_counts, const orc_geom *g, int window,
                            const int *zlist, int nz, double *vol, int nthreads);
/* Half-fan sinogram completion (out [rows][N][2W-1-2am]) and fan->parallel
 * rebinning (out [rows][N/2][2W-1-2am]) in double, for rows independent
 * [N][W] sinograms (rsq_load.cpp:327-470). */
void orc_half2fullfan_f64(const double *in, int W, int N, int rows, int am, double D, double dfi, int flip,
                          double *out);
void orc_half2para_f64(const double *in, int W, int N, int rows, int am, double D, double dfi, double *out);
/* FP64 adjoint of the FDK A = B F W (line integrals -> volume, exact slice
 * centring): out = W F B^T vol, with B^T the transpose of the bilinear
 * backprojection (same masks and weights) and F the symmetric ramp filter.
 * vol [Z][Y][X], out [H][N][W] (double). */
int orc_fdk_adjoint_f64(const float *vol, const orc_geom *g, int window, double *out, int nthreads);
/* The plain backprojection B (FBPConeKernel + fQ3D, kernel.cu:68-177, scale
 * dfi/p of kernel.cu:113, 575) and its exact transpose B^T in double, q as
 * [N][H][W]: the pair of the volume data-consistency refinement. */
int orc_b_f64(const double *q, const orc_geom *g, double *vol, int nthreads);
int orc_bt_f64(const double *vol, const orc_geom *g, double *q, int nthreads);
/* Detector rows [lo, hi] that slices zlist can touch (for sampled oracles). */
void orc_rows_needed(const orc_geom *g, const int *zlist, int nz, int *lo, int *hi);

/* Flat-field + log of raw uint16 intensities as in rsq::FlatFieldCorrection
 * (FBPG/rsq_load.cpp:299-325): v = A*log((I-dark)/(flat-dark)) + B, negated
 * when invert != 0.  dark/flat are per detector pixel [H][W] (per-row in the
 * reference); (I-dark) and (flat-dark) are floored at `floor_counts` so that
 * zero counts give a finite value.  raw layout [N][H][W]; out [H][N][W]. */
void orc_log_u16_f64(const uint16_t *raw, const float *dark, const float *flat,
                     int W, int N, int H, double A, double B, int invert,
                     double floor_counts, float *out_sino, int nthreads);

/* Analytic cone-beam line integrals of a set of ellipsoids.
 * ell: nell records of 16 doubles: centre (3, cm), semi-axes (3, cm),
 * rotation world->local (9, row major), density (1, 1/cm).
 * Coordinates are the volume frame of the backprojector (after axis flips),
 * in cm.  Detector sample (col u, row v) of projection b sits at
 * T = u - cX, Z = v - cZ virtual pixels on the plane through the axis.
 * layout 0: out [H][N][W]; layout 1: out [N][H][W]. */
void orc_project_ellipsoids(const double *ell, int nell, const orc_geom *g, int layout,
                            float *out, int nthreads);

/* Voxelised phantom (density at voxel centres), [nz][Y][X] for zlist. */
void orc_voxelise_ellipsoids(const double *ell, int nell, const orc_geom *g,
                             const int *zlist, int nz, float *vol, int nthreads);

#ifdef __cplusplus
}
#endif
#endif
