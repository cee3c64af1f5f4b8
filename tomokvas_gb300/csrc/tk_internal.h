// tk_internal.h -- host-side interfaces shared by the library's translation units.
#pragma once

#include <cstddef>
#include <cstdint>
#include <cuda_runtime.h>

#include "../../include/tk_fdk.h"

namespace tk {

void set_error(const char *fmt, ...);
int cuda_fail(cudaError_t e, const char *what);

// Row pitch (elements) of the device filtered-projection layout [N][H][Wp]:
// rows start on 16-byte boundaries for every storage precision.
inline int row_pitch(int W) { return (W + 7) & ~7; }
// Coefficient-image row pitch (entries): even, so rows start on 16 bytes.
inline int coef_pitch(int W) { return (W + 1) & ~1; }
inline bool is_coef(int precision) { return precision != TK_F32; }
inline size_t entry_size(int precision)
{
    return precision == TK_F32 ? 4 : precision == TK_F32_COEF ? 16 : 8;
}
inline int storage_pitch(int W, int precision)
{
    return precision == TK_F32 ? row_pitch(W) : precision == TK_F32_COEF ? W : coef_pitch(W);
}
inline size_t filtered_bytes(const tk_geometry &g, int precision)
{
    return (size_t)g.N * (size_t)g.H * (size_t)storage_pitch(g.W, precision) * entry_size(precision);
}
inline bool valid_precision(int p) { return p >= TK_F32 && p <= TK_F32_COEF; }

int validate_geometry(const tk_geometry *g);
int reference_pad_length(int W);

// Angle tables exactly as CalcSinCos builds them (FBPG/kernel.cu:430-441),
// for projections angle0 .. angle0 + g.N - 1.
void build_trig(const tk_geometry &g, float *cos_out, float *sin_out, int angle0 = 0);

// Launchers (asynchronous on `stream`).
// fgrp > 0 (coefficient images from detector frames only): the g.N frames
// come in groups of fgrp, group k at frame k * fstride of d_in and of d_q.
// form: TK_FILTER_FFT or TK_FILTER_TOEPLITZ forces a form (the FFT where the
// Toeplitz product does not support the width); TK_FILTER_AUTO or -1 follows
// filter_form_for.
int launch_filter(const tk_geometry &g, const void *d_in, int input_type, int layout,
                  const tk_flatfield *ff, int window, void *d_q, int precision, float *d_q_scale,
                  cudaStream_t stream, int fgrp = 0, int fstride = 0, int form = -1);
// d_q holds g.N projections whose angle indices start at angle0 (a chunk of
// a longer scan when angle0 > 0).
int launch_backproject(const tk_geometry &g, const void *d_q, int precision, const float *d_q_scale,
                       int nz, float zoff, float *d_vol, int accumulate, cudaStream_t stream, int angle0 = 0);
// The quarter-turn kernel of a coefficient-image format (square centred
// unflipped volume, N divisible by 4, the format's default or selected
// quarter-turn variant): whether it applies, and a launch over
// the quarter-turn images of angles [qbase, qbase + qlen), qbase + qlen <= N/4,
// with d_q holding all N filtered projections, or (compact) only the four
// ranges [qbase + k N/4, + qlen), k = 0..3, one after another.
bool backproject_quarter_ok(const tk_geometry &g, int precision, int nz, float zoff);
int launch_backproject_quarter(const tk_geometry &g, const void *d_q, int precision, const float *d_q_scale, int nz,
                               float zoff, float *d_vol, int accumulate, cudaStream_t stream, int qbase, int qlen,
                               bool compact = false);
int launch_filter_transpose(const tk_geometry &g, const float *d_qbar, int window, float *d_pbar, int layout,
                            cudaStream_t stream);
// The ramp filter as a Toeplitz product on the tensor cores (tk_toeplitz.cu):
// whether a width / storage format / output layout is supported, and the
// launch (after launch_filter has set up the storage scale).  Hf is the float
// spectrum of pad length p the FFT form multiplies by.
struct LoadParams;
bool toeplitz_supported(int W, int precision, int out_layout);
int launch_filter_toeplitz(const LoadParams &L, const float *Hf, int p, void *d_q, int precision,
                           const float *d_q_scale, long long nrows, int pitch, int fgrp, int fstride,
                           cudaStream_t stream);
// The filter form launch_filter runs for a width and storage format under the
// current selection (tk_filter_select_form): TK_FILTER_FFT or TK_FILTER_TOEPLITZ.
int filter_form_for(int W, int precision);
int launch_forward_project(const tk_geometry &g, const float *d_vol, int nz, float zoff, float *d_qbar,
                           int accumulate, cudaStream_t stream);
int launch_phantom(const tk_geometry &g, const double *ell, int nell, int layout, float *d_out,
                   cudaStream_t stream);

// Analytic bound (entries) of the footprint box of a TX x TY x TZ voxel tile
// in any projection, for sample (coef = false) or coefficient storage, with
// the box width rounded to the TMA granularity `align`.
int bp_box_dims(const tk_geometry &g, int nz, float zoff, int TX, int TY, int TZ, bool coef, int align, int *BW,
                int *BH);

// Counts one kernel launch issued by this library (tk_kernel_launches).
void count_launch(unsigned n = 1);

// Device error word of the current device (allocated on first use).
unsigned *device_error_word();

// Backprojection tile configuration (chosen by the autotuner or defaults).
struct BPConfig {
    int variant;  // index into the compiled kernel table
};

}  // namespace tk
