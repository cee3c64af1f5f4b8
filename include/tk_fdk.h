/*
 * tk_fdk.h -- C ABI of the GB300-native FDK cone-beam reconstructor.
 *
 * Drop-in replacement for the GPU engine of Lukas-kV/TomoKvas, class
 * FilteredBackProjection (FBPG/kernel.cuh:82-151, FBPG/kernel.cu:219-897).
 * Every entry point is extern "C", takes plain pointers and sizes, and
 * returns a tk_status; tk_last_error() holds the message of the last
 * failure on the calling thread.  Reference citations are file:line inside
 * the TomoKvas repository.
 *
 * Conventions (identical to the reference):
 *   sinogram-major input  [H][N][W]  (row, angle, column) -- the layout
 *       cra_con::LoadData produces (FBPG/mucat_file.cpp:244-249);
 *   projection-major input [N][H][W] -- the detector frame order of the
 *       .CRA raw file (FBPG/mucat_file.cpp:255-267);
 *   volume [Z][Y][X] float32 (FBPG/kernel.cu:116-117).
 * Filtered projections are kept on the device projection-major.
 */
#ifndef TK_FDK_H
#define TK_FDK_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define TK_FDK_ABI_VERSION 1

typedef enum tk_status {
    TK_OK = 0,
    TK_ERR_INVALID = 1,     /* bad argument or geometry */
    TK_ERR_CUDA = 2,        /* CUDA runtime error (message in tk_last_error) */
    TK_ERR_OOM = 3,         /* device or host allocation failed / over budget */
    TK_ERR_STATE = 4,       /* call out of sequence (e.g. before initialize) */
    TK_ERR_IO = 5,          /* file I/O failure */
    TK_ERR_DEVICE = 6,      /* a kernel reported a failed self-check */
    TK_ERR_UNSUPPORTED = 7  /* valid request the library does not handle */
} tk_status;

typedef enum tk_window {   /* ramp filter apodisation */
    TK_WINDOW_RAMLAK = 0,  /* reference filter: FillFilter/RamLak, kernel.cu:783-802 */
    TK_WINDOW_SHEPP_LOGAN = 1,
    TK_WINDOW_HANN = 2
} tk_window;

/* Storage of the filtered projections between filter and backprojection;
 * all arithmetic stays FP32.
 *   TK_F32       raw FP32 samples, [N][H][Wp], Wp = (W + 7) & ~7         4 B
 *   TK_F16       FP16 bilinear coefficient image, [N][H][Wc],
 *                Wc = (W + 1) & ~1, entry {(Q, dV), (dU, dUV)} as half2 x2  8 B
 *   TK_BF16      the same in bfloat16                                       8 B
 *   TK_F32_COEF  FP32 coefficient image, [N][H][W], entry (Q, dU, dV, dUV) 16 B
 * where for sample q[r][c]: Q = q[r][c], dU = q[r][c+1] - Q,
 * dV = q[r+1][c] - Q, dUV = q[r+1][c+1] - q[r+1][c] - dU (samples outside
 * the detector are zero), so bilinear interpolation inside cell (r, c) is
 * Q + fu dU + fv (dV + fu dUV). */
typedef enum tk_precision {
    TK_F32 = 0,
    TK_F16 = 1,
    TK_BF16 = 2,
    TK_F32_COEF = 3
} tk_precision;

typedef enum tk_layout {
    TK_LAYOUT_SINOGRAM = 0,   /* [H][N][W], reference SetSinogramProperties */
    TK_LAYOUT_PROJECTION = 1  /* [N][H][W], detector frames */
} tk_layout;

typedef enum tk_input {
    TK_INPUT_F32 = 0,  /* line integrals */
    TK_INPUT_U16 = 1   /* raw intensities, log-transformed on the GPU */
} tk_input;

/* Reference parameter set.  Fields map one-to-one onto the arguments of
 * SetSinogramProperties (kernel.cu:479-497), SetReconstructionProperties
 * (kernel.cu:524-537), SetScaleXYZ (kernel.cu:308-311) and SetAxisDirection
 * (kernel.cu:499-507). */
typedef struct tk_geometry {
    int W, N, H;     /* sin_X (columns), sin_Y (angles), sin_Z (rows) */
    float cX, cZ;    /* detector centre: column of the rotation axis, row */
    float dfi;       /* angular step (rad) */
    float D;         /* source-axis distance in virtual pixels */
    float tau;       /* virtual pixel pitch at the axis (cm) */
    int X, Y, Z;     /* volume size */
    float cx, cy, cz;/* volume centre arguments of SetReconstructionProperties */
    float rot;       /* rotation offset (rad) */
    float scale;     /* voxel pitch in virtual pixels */
    int dirx, diry, dirz; /* axis flips */
} tk_geometry;

/* Flat-field + log for raw uint16 input, rsq::FlatFieldCorrection
 * (FBPG/rsq_load.cpp:299-325):
 *   p = A * log((I - dark) / (flat - dark)) + B,  negated when invert != 0.
 * dark/flat are device pointers to [H][W] floats, or NULL to use the scalar.
 * (I - dark) and (flat - dark) are floored at floor_counts (> 0). */
typedef struct tk_flatfield {
    const float *dark;
    const float *flat;
    float dark_value;
    float flat_value;
    float A, B;
    int invert;
    float floor_counts;
} tk_flatfield;

/* ---------------------------------------------------------------- misc */

int tk_version(void);
const char *tk_last_error(void);
/* FilteredBackProjection::GetFreeMemInfo (kernel.cu:313-322). */
size_t tk_get_free_mem_info(int gpu);
/* Pad length of the reference FFT filter, p = 2 * nextpow2(W) (kernel.cu:570-573). */
int tk_pad_length(int W);
/* z offset of a whole-volume backprojection: aZ = scale * (z + zoff). */
float tk_default_zoff(const tk_geometry *g);
/* Per-block z offsets of the reference's Z-block schedule (kernel.cu:398-400,
 * 821).  Writes at most cap offsets; returns the number of blocks. */
int tk_zblock_offsets(const tk_geometry *g, int zb, float *zoff_out, int cap);
/* Reads and (if clear) resets the device-side self-check bits of the current
 * device.  Synchronises the device. */
int tk_device_error_flags(unsigned *flags_out, int clear);

/* ------------------------------------------- stage API (device buffers) */
/* All pointers are device pointers; `stream` is a cudaStream_t (NULL = the
 * legacy default stream).  Calls are asynchronous with respect to the host. */

/* Preprocessing + ramp filter: fuses the uint16 log transform
 * (rsq_load.cpp:299-325), the cosine pre-weight (RB_comma3DKernel,
 * kernel.cu:179-201) and the row-wise ramp filter (fConvolution,
 * kernel.cu:557-781).  Output d_q is projection-major in the storage format
 * `precision` (see tk_precision), with sample values equal to the reference's
 * unnormalised C2R output times the storage scale s.  For the FP32 formats
 * s = 1 and d_q_scale may be NULL.  For 16-bit storage, s is a power of two
 * chosen on the device from the data so that values stay well inside the
 * format's range; it is written to the device float *d_q_scale.  The
 * coefficient formats support W <= 2048. */
int tk_filter_projections(const tk_geometry *g, const void *d_in, int input_type, int layout,
                          const tk_flatfield *ff, int window, void *d_q, int precision,
                          float *d_q_scale, void *stream);

/* Voxel-driven cone-beam backprojection (FBPConeKernel + fQ3D,
 * kernel.cu:68-177) of filtered projections d_q ([N][H][Wp] as written by
 * tk_filter_projections, storage scale in the device float *d_q_scale, or
 * 1 when d_q_scale is NULL) into the slab d_vol[nz][Y][X] whose slices sit
 * at aZ = scale*(z + zoff).  accumulate != 0 adds to the slab
 * (CollectionKernel, kernel.cu:203-215). */
int tk_backproject(const tk_geometry *g, const void *d_q, int precision, const float *d_q_scale,
                   int nz, float zoff, float *d_vol, int accumulate, void *stream);

/* Bytes of the filtered projections in a storage format. */
size_t tk_filtered_bytes(const tk_geometry *g, int precision);
/* Device bytes tk_fdk_device needs as workspace (filtered projections plus
 * a 256-byte header holding the storage scale). */
size_t tk_fdk_workspace_bytes(const tk_geometry *g, int precision);

/* Whole FDK on device buffers: filter into d_workspace, backproject into
 * d_vol[Z][Y][X].  Allocates nothing. */
int tk_fdk_device(const tk_geometry *g, const void *d_in, int input_type, int layout,
                  const tk_flatfield *ff, int window, int precision,
                  void *d_workspace, size_t workspace_bytes, float *d_vol, void *stream);

/* ---------------------------------------------------------- out-of-core
 * Whole FDK with the projections left in host memory (projection-major
 * [N][H][W], TK_INPUT_F32 or TK_INPUT_U16), streamed to the GPU in chunks of
 * `chunk` projections: the host-to-device copy of chunk k+1 (and k+2) runs on
 * a library-owned copy stream while chunk k is filtered and backprojected on
 * `stream`, and the volume d_vol[Z][Y][X] accumulates the chunks.  Page-locked
 * host memory (cudaHostAlloc / cudaHostRegister) lets the copies overlap;
 * pageable memory works but serialises them.  The reference splits the angles
 * into sub-allocations and sums partial volumes ("collecting",
 * kernel.cu:342-371, 849-876); here the volume stays whole in HBM and the
 * projections stream instead.  With FP16 storage on a scan that has the
 * quarter-turn symmetry (square volume centred on the axis, no flips, N
 * divisible by 4), a chunk is instead the four ranges of chunk/4 projections
 * a quarter turn apart, [k chunk/4 + q N/4, + chunk/4), q = 0..3, so that the
 * quarter-turn backprojector runs on every chunk.  Returns once the work is
 * enqueued: h_in must stay valid and unchanged until `stream` has passed it.
 * Allocates nothing on the device (the workspace holds two raw chunks and one
 * filtered chunk). */
size_t tk_fdk_stream_workspace_bytes(const tk_geometry *g, int input_type, int precision, int chunk);
int tk_fdk_stream(const tk_geometry *g, const void *h_in, int input_type, const tk_flatfield *ff, int window,
                  int precision, int chunk, void *d_workspace, size_t workspace_bytes, float *d_vol,
                  void *stream);

/* ------------------------------------------------ adjoint (differentiation)
 * The FDK A = B F W is linear in the line integrals: W the cosine weight
 * (diagonal), F the ramp filter (symmetric Toeplitz: its spectrum is real and
 * even), B the backprojection.  Its transpose A^T = W F B^T gives gradients
 * with respect to the projections.  No counterpart in the reference. */

/* B^T: exact transpose of tk_backproject for TK_F32 storage (same masks,
 * bilinear weights and scale dfi/p).  Scatters d_vol[nz][Y][X] (slices at
 * aZ = scale*(z + zoff)) into d_qbar [N][H][Wp] FP32; accumulate = 0 clears
 * d_qbar first.  FP32 atomics: results are deterministic to rounding only. */
int tk_forward_project(const tk_geometry *g, const float *d_vol, int nz, float zoff, float *d_qbar,
                       int accumulate, void *stream);
/* (F W)^T = W F: filters d_qbar [N][H][Wp] with the ramp of `window` and
 * multiplies by the cosine weight; writes d_pbar FP32 in `layout`. */
int tk_filter_transpose(const tk_geometry *g, const float *d_qbar, int window, float *d_pbar, int layout,
                        void *stream);
/* A: line integrals (FP32, `layout`) -> volume [Z][Y][X]; tk_fdk_device with
 * TK_F32 storage. */
int tk_fdk_forward(const tk_geometry *g, const float *d_proj, int layout, int window, void *d_workspace,
                   size_t workspace_bytes, float *d_vol, void *stream);
/* A^T: volume gradient [Z][Y][X] -> gradient with respect to the line
 * integrals (FP32, `layout`).  Workspace: tk_fdk_workspace_bytes(g, TK_F32). */
int tk_fdk_backward(const tk_geometry *g, const float *d_vol_grad, int layout, int window, void *d_workspace,
                    size_t workspace_bytes, float *d_proj_grad, void *stream);

/* --------------------------------- volume data-consistency refinement
 * Refines a volume x (the FDK volume x0 = B q to start) by gradient steps on
 * the data-consistency loss L(x) = ||B^T x - q||^2,
 *   x <- x - alpha B (B^T x - q),
 * where B is the FP32 backprojection (tk_backproject with TK_F32 samples,
 * FBPConeKernel + fQ3D of kernel.cu:68-177) and B^T its exact transpose
 * (tk_forward_project), and q = F W p the filtered projections of the
 * measured line integrals.  q is the only data a step needs besides x: it is
 * checkpointed once after the filter (tk_refine_checkpoint) as FP32 samples,
 * or as FP16 samples where HBM is short (half the bytes; the residual is
 * formed in FP32).  A step is B^T x, one residual pass (r = -alpha (B^T x - q)
 * and the loss's block partials), and B r accumulated into x; the loss is
 * summed in compensated FP32 when d_loss is given.  alpha < 2 / lambda_max(B B^T)
 * decreases L at every step; tk_refine_step_size returns 1 / lambda_max from a
 * power iteration.  The workspace (tk_refine_workspace_bytes, 256-byte
 * aligned) holds the FP32 residual and the partial sums.  No counterpart in the
 * reference, which stops at the FDK volume. */
size_t tk_refine_checkpoint_bytes(const tk_geometry *g, int precision); /* TK_F32 or TK_F16 samples [N][H][Wp] */
size_t tk_refine_workspace_bytes(const tk_geometry *g);
/* q = F W p (the FFT filter of the FP32 FDK) into d_ckpt [N][H][Wp]. */
int tk_refine_checkpoint(const tk_geometry *g, const void *d_in, int input_type, int layout,
                         const tk_flatfield *ff, int window, void *d_ckpt, int precision,
                         void *d_workspace, size_t workspace_bytes, void *stream);
/* `steps` gradient steps on d_vol[Z][Y][X] in place; d_loss (device, may be
 * NULL) receives L(x_k) before step k for k < steps. */
int tk_refine_volume(const tk_geometry *g, const void *d_ckpt, int precision, float alpha, int steps,
                     float *d_vol, double *d_loss, void *d_workspace, size_t workspace_bytes, void *stream);
/* 1 / lambda_max(B B^T) by `iters` power iterations from a fixed
 * pseudo-random volume (d_vol_tmp, overwritten).  Synchronous. */
int tk_refine_step_size(const tk_geometry *g, int iters, float *d_vol_tmp, void *d_workspace,
                        size_t workspace_bytes, float *alpha_out, void *stream);

/* Whole FDK on device buffers for callers that cannot allocate device memory:
 * a service that reserves a fixed device-memory budget at start-up and may
 * not grow it, or code inside a callback or timing-critical loop where
 * cudaMalloc's implicit device synchronisation and possible failure are not
 * acceptable.  Same work and results as tk_fdk_device, but the workspace is a
 * static device array of 64 MiB inside the library, so the problem must fit
 * it: tk_fdk_workspace_bytes(g, precision) <= 64 MiB (for example 180
 * projections of 256 x 256 in TK_F32); larger problems are rejected with
 * TK_ERR_UNSUPPORTED and a message.  The caller still passes the input and
 * the output volume.  Every GPU that loads the library holds the array until
 * the process exits.  The first call on a device looks the array up (with
 * that device current) and, with lazy module loading, loads the kernels it
 * runs: make one warm-up call per device before fixing the memory budget or
 * starting a stream capture.  A cudaDeviceReset after it invalidates the
 * looked-up address.  All calls share the array: calls that overlap on the
 * GPU race and must be serialised.  Allocates no device memory (the first call
 * with a new filter setting fills a host-side cache of its spectrum).  No
 * counterpart in the reference. */
int tk_fdk_device_noalloc(const tk_geometry *g, const void *d_in, int input_type, int layout,
                          const tk_flatfield *ff, int window, int precision, float *d_vol, void *stream);

/* Ramp-filter form.  The filter is the convolution of each detector row with
 * the even kernel K = C2R_p(tau |R2C_p(h)|), a symmetric Toeplitz matrix
 * (fConvolution, kernel.cu:557-781):
 *   TK_FILTER_FFT       shared-memory Stockham FFT of the padded row (any W);
 *   TK_FILTER_TOEPLITZ  the W x W Toeplitz product on the tcgen05 tensor
 *                       cores with split-BF16 compensated products and FP32
 *                       accumulation (8 <= W <= 512; other widths take the FFT);
 *   TK_FILTER_AUTO      (default) the Toeplitz product for 16-bit storage
 *                       up to W = 512, where it is the faster form; the FFT
 *                       for wider rows and for FP32 storage (the split-BF16
 *                       product carries about 2e-5 relative error, below
 *                       16-bit rounding but above the FP32 forms' bound).
 * The selection is process-wide; tk_filter_form_for reports the form a width and
 * storage format would run.  No counterpart in the reference (cuFFT only). */
typedef enum tk_filter_form {
    TK_FILTER_AUTO = 0,
    TK_FILTER_FFT = 1,
    TK_FILTER_TOEPLITZ = 2
} tk_filter_form;
int tk_filter_select_form(int form);
int tk_filter_form_for(int W, int precision);

/* Backprojection kernel variants (tile shape, pipeline), for benchmarking
 * and the autotuner; no counterpart in the reference, whose launch shape is
 * fixed (kernel.cu:825-827).  tk_bp_select_variant(-1) restores the default
 * choice; a selected variant applies to launches of its storage precision. */
int tk_bp_variant_count(void);
const char *tk_bp_variant_name(int i);
int tk_bp_variant_precision(int i);
int tk_bp_select_variant(int i);
/* Forward projector (the scatter of tk_forward_project / tk_fdk_backward):
 * 0 (default) lanes on 32 consecutive slices of one voxel column, the warp
 * walking its columns, accumulating each projection's box in two-word fixed
 * point with integer shared atomics (2^-25 or finer of the tile's largest
 * contribution; FP32 atomics when the source lies inside the field of view);
 * 1 lanes on 32 voxel columns, each walking its slices (FP32 shared
 * atomics); 2 the slice-lane form with FP32 shared atomics.  Same weights
 * and masks; the sums differ by FP32 rounding only.  The fixed-point form
 * expects finite volume values. */
int tk_fp_select_variant(int i);

/* Analytic cone-beam line integrals of ellipsoids (seeded synthetic input).
 * ell: host array of nell records of 16 doubles: centre[3] (cm), semi-axes[3]
 * (cm), rotation world->local[9], density (1/cm).  Output device float
 * array in `layout`. */
int tk_phantom_project(const tk_geometry *g, const double *ell, int nell, int layout,
                       float *d_out, void *stream);

/* ------------------------------------------------ fan-beam rsq helpers
 * Offset-detector (half-fan) sinogram completion and fan->parallel
 * rebinning of `rows` independent fan-beam sinograms d_in [rows][N][W]
 * (FP32) with the rotation axis at column axis_move, source distance D
 * (pixels, D > W) and angle step dfi (a full 360-degree scan):
 * rsq::Half2FullFan (FBPG/rsq_load.cpp:327-380) writes d_out
 * [rows][N][2W-1-2 axis_move] (flip: angles in reverse order);
 * rsq::Half2Para / Fan2Para (FBPG/rsq_load.cpp:382-470) writes d_out
 * [rows][N/2][2W-1-2 axis_move].  Asynchronous on `stream`. */
int tk_half_to_full_fan(const float *d_in, int W, int N, int rows, int axis_move, double D, double dfi, int flip,
                        float *d_out, void *stream);
int tk_half_to_parallel(const float *d_in, int W, int N, int rows, int axis_move, double D, double dfi,
                        float *d_out, void *stream);

/* ---------------------------------------------------------------- batches
 * Many independent reconstructions of uneven detector, angle and volume sizes
 * in one persistent backprojection launch.  Submit items (device input,
 * output volume, geometry, filter), plan them onto one device workspace, then
 * run: each item is filtered (one launch per item), then ONE persistent
 * kernel backprojects the voxel tiles of all items, taken from a shared work
 * counter, larger items first (items with the quarter-turn symmetry instead
 * get tk_fdk_device's quarter-turn launch beside it, tk_batch_item_quarter_turn).  tk_batch_run(use_graph = 1) captures the run
 * into a CUDA graph on first use and replays it afterwards (inputs are read
 * from the submitted pointers at every run).  tk_batch_autotune times every
 * compiled tile shape of the batch's storage format on the planned batch and
 * keeps the fastest, after choosing each item's filter form (FFT or tensor-core
 * Toeplitz product) by timing both.  Storage is a coefficient image (TK_F16 by default, or
 * TK_BF16 / TK_F32_COEF); W <= 2048.  Results equal tk_fdk_device's for the
 * same tile shape.  No counterpart in the reference (one volume per process).
 * A batch is not thread-safe; submitted buffers must outlive its runs. */
typedef struct tk_batch tk_batch;
int tk_batch_create(tk_batch **out);
void tk_batch_destroy(tk_batch *b);
int tk_batch_set_precision(tk_batch *b, int precision);
/* Adds one item (index = tk_batch_size(b) - 1 after success). */
int tk_batch_submit(tk_batch *b, const tk_geometry *g, const void *d_in, int input_type, int layout,
                    const tk_flatfield *ff, int window, float *d_vol);
int tk_batch_size(const tk_batch *b);
size_t tk_batch_workspace_bytes(tk_batch *b);
/* Lays out the workspace (256-byte aligned) and uploads the item tables;
 * synchronises `stream`. */
int tk_batch_plan(tk_batch *b, void *d_workspace, size_t workspace_bytes, void *stream);
int tk_batch_run(tk_batch *b, int use_graph, void *stream);
/* Times each tile shape of the storage format (3 runs each) and keeps the
 * fastest; writes its index and time per run (ms).  Synchronous. */
int tk_batch_autotune(tk_batch *b, void *stream, int *variant_out, float *ms_out);
int tk_batch_variant_count(void);
const char *tk_batch_variant_name(int i);
/* The tile shape the planned batch uses (-1 before planning). */
int tk_batch_variant(const tk_batch *b);
/* Forces a tile shape (-1: default); takes effect at the next plan. */
int tk_batch_select_variant(tk_batch *b, int i);
/* The filter form item i runs (tk_filter_form): TK_FILTER_AUTO until
 * tk_batch_autotune, which times both forms on each item and keeps the faster
 * (the tensor-core Toeplitz product only where it supports the width); -1 for
 * a bad index. */
int tk_batch_item_filter_form(const tk_batch *b, int i);
/* 1 when item i of the planned batch has the quarter-turn symmetry that
 * tk_fdk_device's quarter-turn kernel needs (square centred unflipped volume,
 * N divisible by 4, the storage format's quarter-turn variant selected or
 * default): such items are backprojected by that same launch, on their filter
 * stream beside the persistent kernel, with the per-volume bits; 0 for items
 * of the persistent kernel; -1 for a bad index or an unplanned batch. */
int tk_batch_item_quarter_turn(const tk_batch *b, int i);
/* Phase times of the last eager tk_batch_run (use_graph = 0): from the run's
 * start until every item's filter has finished, and the backprojection after
 * it (the persistent launch and the quarter-turn items' launches; waits for
 * that run to finish). */
int tk_batch_timings(tk_batch *b, float *filter_ms, float *bp_ms);

/* ------------------------------------------------------------ diagnostics
 * tk_kernel_launches: kernels this library has launched in this process (a
 * monotonic count, for measuring how many launches a region issued).
 * tk_measure_fp32_fma_rate: times a bounded FP32 FMA throughput kernel on the
 * current device (about a millisecond) and writes its rate in TFLOP/s, the
 * FP32-pipe ceiling the backprojection is measured against.  Synchronous. */
unsigned long long tk_kernel_launches(void);
int tk_measure_fp32_fma_rate(double *tflops_out);
/* Self-check exercises (tests of the failure reporting; nothing faults):
 * tk_diag_wait_timeout launches one CTA that waits, with the library's bounded
 * wait and the given limit, on an mbarrier armed for copies that are never
 * issued; it leaves ERR_WAIT_TIMEOUT (0x2) in the device error word, read by
 * tk_device_error_flags.  tk_diag_shrink_box(rows) takes `rows` rows off the
 * staged footprint box of every per-volume backprojection launch (tk_backproject,
 * tk_fdk_device, the handle) from then on (0 restores it): the
 * kernels' bounds checks then skip the reads that fall outside and report
 * ERR_BOX_OVERFLOW (0x1), which the handle returns as TK_ERR_DEVICE. */
int tk_diag_wait_timeout(double limit_ms, void *stream);
int tk_diag_shrink_box(int rows);

/* ------------------------------ FilteredBackProjection mirror (handle) */
/* One handle = one FilteredBackProjection object (kernel.cuh:82-151).
 * Call order as in FBPG/para_TC.cpp:130-153: setters -> initialize ->
 * calculate_reconstruction -> destroy.  The host sinogram passed to
 * set_sinogram_properties is borrowed until tk_fdk_initialize returns. */

typedef struct tk_fdk tk_fdk;

/* bin_siz::GetBlock(block, collecting) (FBPG/mucat_file.cpp:576-642): returns
 * a host buffer of X*Y*ZB floats for Z block `block`.  When `collecting` is
 * set the buffer already holds the partial volume of earlier angle blocks
 * and the engine adds its result to it.  Calling the sink for block n
 * releases the buffer of block n-1.  NULL aborts the reconstruction. */
typedef float *(*tk_block_sink)(void *user, int block, int collecting);

int tk_fdk_create(tk_fdk **out);                                   /* kernel.cu:219-253 */
void tk_fdk_destroy(tk_fdk *h);                                    /* kernel.cu:255-281, no device reset */
int tk_fdk_set_gpu_id(tk_fdk *h, int id);                          /* SetGPUid kernel.cu:283-286 */
int tk_fdk_set_block_size(tk_fdk *h, int zb);                      /* SetBlockSize kernel.cu:288-291 */
int tk_fdk_set_allocation_limit(tk_fdk *h, long long bytes);       /* SetAllocationLimit kernel.cu:303-306 */
int tk_fdk_set_collecting(tk_fdk *h, int collecting);              /* SetCollecting kernel.cu:293-296 */
int tk_fdk_set_show_info(tk_fdk *h, int show);                     /* SetShowInfo kernel.cu:298-301 */
int tk_fdk_set_axis_direction(tk_fdk *h, int x, int y, int z);     /* SetAxisDirection kernel.cu:499-507 */
int tk_fdk_show_info(tk_fdk *h);                                   /* fShowInfo kernel.cu:901-913, on stdout */
int tk_fdk_set_sinogram_properties(tk_fdk *h, const float *sinogram, int W, float cX, int N, int H,
                                   float cZ, float dfi, float D, float tau); /* kernel.cu:479-497 */
int tk_fdk_set_reconstruction_properties(tk_fdk *h, int X, float cx, int Y, float cy, int Z, float cz,
                                         float rot);               /* kernel.cu:524-537 */
int tk_fdk_set_scale_xyz(tk_fdk *h, float scale);                  /* SetScaleXYZ kernel.cu:308-311 */
/* Extensions with no reference setter. */
int tk_fdk_set_projections_u16(tk_fdk *h, const uint16_t *raw, int layout, const float *dark_hw,
                               const float *flat_hw, float dark_value, float flat_value, float A, float B,
                               int invert, float floor_counts);   /* rsq_load.cpp:299-325 */
int tk_fdk_set_input_layout(tk_fdk *h, int layout);
int tk_fdk_set_filter(tk_fdk *h, int window);
int tk_fdk_set_precision(tk_fdk *h, int precision);
int tk_fdk_set_stream(tk_fdk *h, void *stream);
/* Pipelined mode (off by default; the C++ FilteredBackProjection turns it on).
 * tk_fdk_initialize uploads the projections in chunks of N/8 angles, filters
 * each chunk as it lands and backprojects the chunks of the first quarter of
 * the angles into a whole-volume device buffer (Z block by Z block, the
 * reference's block offsets) as they land; it then queues one accumulating
 * launch per Z block over the rest (the last block's in two parts) and
 * returns once the host buffer has been read.  With FP16 storage on a scan
 * with the quarter-turn symmetry (square volume centred on the axis, no flips,
 * N divisible by 4) the chunks are sets of four angle ranges a quarter turn
 * apart, filtered on their own stream, and one launch backprojects the first
 * quarter to third of the angles once they are filtered.
 * tk_fdk_calculate_reconstruction only delivers the blocks, each copy starting
 * once its block's launch has run, overlapping the next block's launch.  It applies to
 * non-collecting runs with N >= 128 whose storage scale is known up front
 * (FP32 storage, or uint16 counts with scalar flat/dark) and whose volume fits
 * in device memory beside the projections; otherwise the regular path runs.
 * The chunk sums change FP32 rounding only.  A setter called after
 * initialize drops the pipelined volume; tk_fdk_reconstruct_device always
 * computes its own. */
int tk_fdk_set_pipeline(tk_fdk *h, int on);
/* Initialize (kernel.cu:324-428): select the device, allocate, copy the
 * projections to the GPU, build the angle tables. */
int tk_fdk_initialize(tk_fdk *h);
/* CalculateReconstruction (kernel.cu:804-897): filter, then backproject Z
 * block by Z block and hand every block to the sink, exactly following the
 * reference's block schedule (including its last-slice quirk). */
int tk_fdk_calculate_reconstruction(tk_fdk *h, tk_block_sink sink, void *user);
/* Whole volume into a device buffer d_vol[Z][Y][X] (all Z slices). */
int tk_fdk_reconstruct_device(tk_fdk *h, float *d_vol);
/* Milliseconds spent in the stages of the last initialize + reconstruction,
 * measured with CUDA events: the filter, the backprojection (filter and
 * backprojection together in the pipelined mode, where they interleave), the
 * upload, and d2h_ms, the part of the block copies to the host that runs after
 * the last backprojection (the copies before it overlap the computation). */
int tk_fdk_get_timings(tk_fdk *h, float *filter_ms, float *bp_ms, float *h2d_ms, float *d2h_ms);

#ifdef __cplusplus
}
#endif
#endif /* TK_FDK_H */
