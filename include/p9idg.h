/*
 * p9idg.h -- C ABI of the GB300 (sm_103a) image-domain gridder with w-stacking.
 *
 * Drop-in for the gridding path of lord-blueberry/p9-distributed-reconstruction
 * (C#, project "Core", namespace Core.ImageDomainGridder).  Every entry point
 * names the reference member it replaces (file:line, paths inside
 * Distributed-Reconstruction/).  A C# caller binds these with P/Invoke; the
 * arrays it passes are its own pinned, row-major multidimensional arrays:
 *
 *   double[nbl, nt, 3]      uvw          metres
 *   double[nch]             frequencies  Hz
 *   Complex[nbl, nt, nch]   vis          interleaved (re, im) doubles
 *   bool[nbl, nt, nch]      flags        one byte per sample, nonzero = flagged
 *   Complex[N, N]           grid         interleaved (re, im) doubles
 *   List<Complex[N, N]>     w layers     passed as one [W][N][N] block
 *
 * Callers own every array.  The library owns plans, device memory, CUDA
 * streams and cuFFT plans.  Calls on distinct plans may run from different
 * threads; a single plan is not re-entrant.  All entry points return a status;
 * p9idg_last_error() gives a thread-local message for the last failure.
 */
#ifndef P9IDG_H
#define P9IDG_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef int32_t p9idg_status;

enum {
    P9IDG_OK = 0,
    P9IDG_INVALID_ARGUMENT = 1,     /* bad sizes/pointers; also the reference's IndexOutOfRange cases */
    P9IDG_CANNOT_PLACE = 2,         /* "could not place (all) visibilities on subgrid" Partitioner.cs:86,91 */
    P9IDG_SUBGRID_OUT_OF_GRID = 3,  /* "subgrid falls not within grid" Partitioner.cs:118 */
    P9IDG_INVALID_GRID = 4,         /* "invalid grid" Adder.cs:49 */
    P9IDG_OUT_OF_MEMORY = 5,
    P9IDG_CUDA_ERROR = 6,
    P9IDG_NO_DEVICE = 7,
    P9IDG_UNSUPPORTED = 8,          /* e.g. tensor-core mode for a subgrid size it does not cover */
    P9IDG_DEVICE_CHECK_FAILED = 9   /* a kernel's own bounds check tripped (no access was made) */
};

/* Gridding precision of the gridder/degridder kernels.  The FP32 kernels take subgrid sizes 8, 16,
 * 24, 32 and 48; the tensor-core kernels 8, 16, 24 and 32 (a subgrid of S < 32 runs padded to 32
 * operand rows, so it costs what S = 32 costs per visibility). */
enum {
    P9IDG_MODE_FP32 = 0,      /* FP32 sincos + FMA, FP64 per-visibility phase argument */
    P9IDG_MODE_TC_BF16X3 = 1, /* tensor cores, BF16 hi+lo split (3 products), FP32 accumulation */
    P9IDG_MODE_TC_FP16X3 = 2  /* tensor cores, FP16 hi+lo split (3 products), FP32 accumulation */
};

/* Largest |dw * r(x, y)| the tensor-core modes accept.  They write the reference's phasor
 * exp(i dw n(x, y)) (Gridder.cs:61-67) as A(x) B(y) exp(i dw r(x, y)), with r the non-separable
 * remainder of the n table (centred on zero), and expand the last factor in powers of dw r.
 * First-order form up to P9IDG_TC_MAX_W_TERM: the term left out is at most (dw r)^2 / 2 = 5e-5 of
 * each visibility's contribution.  Second-order form (two more operand rows per visibility and a third
 * accumulator block; gridder 12 %, degridder 14 % slower) up to P9IDG_TC_MAX_W_TERM2: the term left out is at most (dw r)^3 / 6 = 4.5e-6.
 * Both stay inside the modes' stated 1e-4 relative-L2 bound together with their rounding.  A
 * plan picks the first-order form where it holds, else the second-order one
 * (p9idg_plan_info.tc_order); a plan beyond P9IDG_TC_MAX_W_TERM2 keeps the FP32 kernels when a
 * tensor-core mode is selected (p9idg_plan_set_mode returns P9IDG_OK, p9idg_plan_info.mode stays
 * P9IDG_MODE_FP32 and p9idg_last_error() says why); a call whose uvw exceeds its plan's form
 * returns P9IDG_UNSUPPORTED. */
#define P9IDG_TC_MAX_W_TERM 0.01
#define P9IDG_TC_MAX_W_TERM2 0.03

/* GriddingConstants (Core/ImageDomainGridder/GriddingConstants.cs:33-52).
 * scale_arcsec is the cell size in radians, stored as float like the
 * reference's ScaleArcSec.  WStepLambda is not a field: the reference never
 * assigns it (GriddingConstants.cs:25), so the w offset of every subgrid is 0.
 * The subgrid taper (SubgridSpheroidal) is the identity unless
 * p9idg_plan_set_taper installs one. */
typedef struct p9idg_params {
    int64_t vis_count;      /* VisibilitiesCount: normalisation of the image FFTs */
    int32_t grid_size;      /* GridSize N */
    int32_t subgrid_size;   /* SubgridSize S */
    int32_t kernel_size;    /* KernelSize (partitioner margin) */
    int32_t max_timesteps;  /* MaxTimestepsPerSubgrid */
    float scale_arcsec;     /* ScaleArcSec (radians per cell) */
    int32_t wlayer_count;   /* WLayerCount */
    double wstep;           /* WStep (wavelengths per w layer; 0 = no w binning) */
} p9idg_params;

/* Subgrid (Core/ImageDomainGridder/Subgrid.cs:15-24).  baseline_idx is the
 * index of the baseline list the subgrid belongs to; the reference gridder
 * indexes uvw/vis with that list index (Gridder.cs:28,58). */
typedef struct p9idg_subgrid {
    int32_t baseline_idx;
    int32_t time_sample_start;
    int32_t time_sample_count;
    int32_t u_pixel;
    int32_t v_pixel;
    int32_t w_lambda;       /* w layer index (may be negative) */
} p9idg_subgrid;

typedef struct p9idg_plan p9idg_plan;

/* Summary of a plan (counts over the subgrid list). */
typedef struct p9idg_plan_info {
    int64_t num_subgrids;
    int64_t input_visibilities;    /* nbl * nt * nch */
    int64_t gridded_visibilities;  /* visibilities covered by subgrids (the partitioner drops some) */
    int64_t work_items;            /* (subgrid, time-chunk) units the gridder kernels process */
    int32_t nbl, nt, nch;
    int32_t mode;                  /* the kernels the plan runs (P9IDG_MODE_*) */
    int32_t requested_mode;        /* the mode last passed to p9idg_plan_set_mode */
    double tc_w_term;              /* max |dw| * max |r| of the plan's samples (vs P9IDG_TC_MAX_W_TERM);
                                      -1 until a tensor-core mode has been requested */
    int32_t tc_order;              /* tensor-core form the plan runs: 1 or 2; 0 when it runs FP32 */
    int32_t reserved;
} p9idg_plan_info;

/* ---------------- plans: Partitioner ---------------- */

/* Partitioner.CreatePartition (Core/ImageDomainGridder/Partitioner.cs:20-125).
 * Builds the subgrid list on the host (bit-identical to the reference's
 * integer output) and uploads uvw, frequencies and the work list to the GPU. */
p9idg_status p9idg_plan_create(const p9idg_params *c, const double *uvw, int32_t nbl, int32_t nt,
                               const double *frequencies, int32_t nch, p9idg_plan **out);

/* A plan from a caller-built List<List<Subgrid>> flattened in list order
 * (the shape IDG.Grid/DeGrid/GridW/DeGridW receive, IDG.cs:12,22,32,42). */
p9idg_status p9idg_plan_create_from_subgrids(const p9idg_params *c, const p9idg_subgrid *subgrids, int64_t nsub,
                                             const double *uvw, int32_t nbl, int32_t nt,
                                             const double *frequencies, int32_t nch, p9idg_plan **out);

p9idg_status p9idg_plan_num_subgrids(const p9idg_plan *plan, int64_t *n);
/* Copies the subgrid list (reference order: baseline-major, then time). */
p9idg_status p9idg_plan_get_subgrids(const p9idg_plan *plan, p9idg_subgrid *out, int64_t capacity);
p9idg_status p9idg_plan_get_info(const p9idg_plan *plan, p9idg_plan_info *out);
/* Selects the gridder/degridder kernels (P9IDG_MODE_*).  A tensor-core mode on a plan whose
 * w term exceeds P9IDG_TC_MAX_W_TERM keeps the FP32 kernels (see there). */
p9idg_status p9idg_plan_set_mode(p9idg_plan *plan, int32_t mode);
/* Tensor-core form: 0 (default) = the first-order form where P9IDG_TC_MAX_W_TERM holds, else the
 * second-order one; 2 = always the second-order form (smaller error, slower).  No counterpart in
 * the reference. */
p9idg_status p9idg_plan_set_tc_order(p9idg_plan *plan, int32_t order);
/* Subgrid taper float[S][S] applied by gridder and degridder (GriddingConstants.SubgridSpheroidal,
 * Gridder.cs:76,111); NULL restores the identity taper the reference uses. */
p9idg_status p9idg_plan_set_taper(p9idg_plan *plan, const float *taper);
/* Runs the plan's work on a caller's cudaStream_t (NULL = the plan's own stream). */
p9idg_status p9idg_plan_set_stream(p9idg_plan *plan, void *cuda_stream);
p9idg_status p9idg_plan_get_stream(const p9idg_plan *plan, void **cuda_stream);
/* The GriddingConstants the plan was made with. */
p9idg_status p9idg_plan_get_params(const p9idg_plan *plan, p9idg_params *out);
/* Creates the plan's device state (stream, constant tables) on the current device now; the
 * device entry points otherwise do this on first use. */
p9idg_status p9idg_plan_init_device(p9idg_plan *plan);
/* Host-array calls (p9idg_grid*, p9idg_degrid*): in_place = 1 (default) lets the kernels read the
 * caller's visibilities and grid and write the degridded visibilities directly in host memory
 * where the device reaches host memory through the host's page tables (NVLink-C2C on Grace),
 * overlapping the link with the kernels; 0 stages every array through device copies.
 * _get reports what the calls will do on this device (1 = in place). */
p9idg_status p9idg_plan_set_host_access(p9idg_plan *plan, int32_t in_place);
p9idg_status p9idg_plan_get_host_access(p9idg_plan *plan, int32_t *in_place);
void p9idg_plan_destroy(p9idg_plan *plan);

/* ---------------- IDG facade, host arrays (Core/ImageDomainGridder/IDG.cs) ---------------- */
/* Every array is sized from the plan (vis and flags [nbl][nt][nch], uvw [nbl][nt][3], grids
 * [N][N], layers [W][N][N]) and must hold that many elements: the library cannot see the
 * caller's array bounds, and with in-place host access (p9idg_plan_set_host_access) the kernels
 * read and write the arrays themselves.  The P/Invoke shim checks GetLength() against the plan. */
/* uvw may be NULL to reuse the uvw the plan was created with. */

/* IDG.Grid (IDG.cs:12-20): Gridder.Forward, SubgridFFT.Forward, Adder.Add, FFT.Shift.  grid_out Complex[N,N]. */
p9idg_status p9idg_grid(p9idg_plan *plan, const double *vis, const double *uvw, double *grid_out);
/* IDG.DeGrid (IDG.cs:22-30).  Like the reference, FFT.Shift is applied to grid_io in place. */
p9idg_status p9idg_degrid(p9idg_plan *plan, double *grid_io, const double *uvw, double *vis_out);
/* IDG.GridW (IDG.cs:32-40): AdderWStack.Add into W layers, each FFT.Shift-ed.  layers_out Complex[W][N,N]. */
p9idg_status p9idg_grid_w(p9idg_plan *plan, const double *vis, const double *uvw, double *layers_out);
/* IDG.DeGridW (IDG.cs:42-50).  FFT.Shift is applied to grid_io in place. */
p9idg_status p9idg_degrid_w(p9idg_plan *plan, double *grid_io, const double *uvw, double *vis_out);
/* IDG.GridPSF (IDG.cs:52-66): IDG.Grid of unit visibilities where not flagged. */
p9idg_status p9idg_grid_psf(p9idg_plan *plan, const double *uvw, const uint8_t *flags, double *grid_out);
/* IDG.ToImage (IDG.cs:68-83): Grid, FFT.Backward(grid, VisibilitiesCount), FFT.Shift.  image_out double[N,N]. */
p9idg_status p9idg_to_image(p9idg_plan *plan, const double *vis, const double *uvw, double *image_out);
/* IDG.CalculatePSF (IDG.cs:85-114). */
p9idg_status p9idg_calculate_psf(p9idg_plan *plan, const double *uvw, const uint8_t *flags, double *psf_out);

/* ---------------- FFT.cs, host arrays (Core/FFT.cs) ---------------- */

/* FFT.WStackIFFTFloat (FFT.cs:188-215): sum over layers of Re(IFFT(layer)) / visCount, float[N,N]. */
p9idg_status p9idg_wstack_ifft_float(const double *layers, int32_t nlayers, int32_t n, int64_t vis_count,
                                     float *image_out);
/* FFT.Forward(float[,] image, double norm) (FFT.cs:99-117): unnormalised forward FFT / norm. */
p9idg_status p9idg_fft_forward_float(const float *image, int32_t n, double norm, double *grid_out);
/* FFT.BackwardFloat(Complex[,] image, double norm) (FFT.cs:139-157): Re(IFFT) / norm. */
p9idg_status p9idg_fft_backward_float(const double *grid, int32_t n, double norm, float *image_out);
/* FFT.Shift (FFT.cs:221-264): in-place quadrant swap of a square [n][n] array, elem_bytes 4, 8 or 16. */
p9idg_status p9idg_fft_shift(void *array, int32_t n, int32_t elem_bytes);

/* ---------------- device-resident interface (HBM buffers, complex64 = float2) ---------------- */
/* These run asynchronously on the plan's stream; p9idg_synchronize waits and
 * reports kernel-side check failures.  uvw and frequencies are the plan's.  The zeroing of an
 * output runs on a second stream of the plan, forked from the plan's stream and joined back into
 * it within the call, so all of a call's work is ordered on the plan's stream. */

/* Gridder + subgrid IFFT + w-stack adder: vis complex64[nbl][nt][nch] -> layers complex64[W][N][N]
 * (already FFT.Shift-ed, as IDG.GridW returns them).  The layers are overwritten. */
p9idg_status p9idg_grid_w_device(p9idg_plan *plan, const void *d_vis, void *d_layers);
/* Splitter + subgrid FFT + degridder: grid complex64[N][N] as passed to IDG.DeGridW (not shifted;
 * the shift is folded into the splitter and the device grid is left unchanged) -> vis complex64. */
p9idg_status p9idg_degrid_w_device(p9idg_plan *plan, const void *d_grid, void *d_vis);
/* Non-w variants (IDG.Grid / IDG.DeGrid): one complex64[N][N] grid. */
p9idg_status p9idg_grid_device(p9idg_plan *plan, const void *d_vis, void *d_grid);
p9idg_status p9idg_degrid_device(p9idg_plan *plan, const void *d_grid, void *d_vis);
/* FFT.WStackIFFTFloat (+ the caller's FFT.Shift when shift != 0) on device layers: float image[N][N]. */
p9idg_status p9idg_wstack_image_device(p9idg_plan *plan, const void *d_layers, float *d_image, int32_t shift);
p9idg_status p9idg_synchronize(p9idg_plan *plan);

/* No counterpart in the reference.  W-stacked gridding (the work of p9idg_grid_w_device, FP32
 * kernels) for callers that cannot allocate device memory: a pipeline that reserves all of its
 * memory up front and forbids allocation afterwards, a framework whose allocator owns every
 * device byte, or a process under a hard device-memory quota.  It takes no plan and calls no
 * allocator; its working memory is one fixed 32 MiB array in the library's device image, which
 * every GPU that loads the library holds until the process exits.
 *   d_subgrids  device array of nsub subgrids (e.g. p9idg_plan_get_subgrids copied to the GPU)
 *   d_uvw       device double[nbl][nt][3];  frequencies: host double[nch], nch <= 64
 *   d_vis       device complex64[nbl][nt][nch];  d_layers: device complex64[W][N][N], overwritten
 * Subgrid sizes 8, 16, 24, 32, 48 only.  Synchronous: returns after the GPU work on cuda_stream
 * (NULL = legacy default stream) has finished.  The first call on a device looks up the array's
 * address; make it before any stream capture.  Under CUDA's lazy module loading (the default,
 * CUDA_MODULE_LOADING=LAZY) the array is committed on a device by that first call, not when the
 * library loads: a caller with a fixed start-up reservation makes one warm-up call then (nsub = 0
 * only clears d_layers).  All calls share the array: calls whose GPU work overlaps race and must
 * be ordered by the caller. */
p9idg_status p9idg_grid_w_device_noalloc(const p9idg_params *c, const p9idg_subgrid *d_subgrids, int64_t nsub,
                                         const double *d_uvw, int32_t nbl, int32_t nt, const double *frequencies,
                                         int32_t nch, const void *d_vis, void *d_layers, void *cuda_stream);

/* ---------------- batches of independent problems (no counterpart in the reference) ---------------- */
/* Many plans (imaging problems of different sizes) gridded and degridded together: every
 * kernel stage is ONE launch over the work items of all problems, ordered largest first, so
 * small problems fill the GPU alongside large ones.  Buffers are the per-problem device
 * buffers of p9idg_grid_w_device / p9idg_degrid_w_device (complex64), fixed at creation.
 * All plans must share the precision mode; they may mix subgrid sizes (one launch per kernel
 * stage and size). */
typedef struct p9idg_batch p9idg_batch;

/* Work-item sizes (visibilities per gridder / degridder item; 0 = default: FP32 1024 / 512,
 * tensor core 4096 / 16384) -- the time-chunk length the autotuner chooses. */
p9idg_status p9idg_plan_set_chunking(p9idg_plan *plan, int32_t gridder_max_vis, int32_t degridder_max_vis);
p9idg_status p9idg_batch_create(p9idg_plan *const *plans, int32_t nplans, const void *const *d_vis,
                                void *const *d_layers, const void *const *d_grids, void *const *d_vis_out,
                                p9idg_batch **out);
/* IDG.GridW / IDG.DeGridW for every problem of the batch (asynchronous, on the batch's stream). */
p9idg_status p9idg_batch_grid_w(p9idg_batch *batch);
p9idg_status p9idg_batch_degrid_w(p9idg_batch *batch);
/* Records grid_w + degrid_w into a CUDA graph; later p9idg_batch_run calls replay it. */
p9idg_status p9idg_batch_capture_graph(p9idg_batch *batch);
/* grid_w then degrid_w (graph replay once captured). */
p9idg_status p9idg_batch_run(p9idg_batch *batch);
/* Launch order of the work items: THROUGHPUT (default) interleaves all problems largest item
 * first; SMALL_FIRST runs the problems in order of size so the small ones finish early in each
 * phase.  Drops a captured graph (capture again). */
enum { P9IDG_SCHEDULE_THROUGHPUT = 0, P9IDG_SCHEDULE_SMALL_FIRST = 1 };
p9idg_status p9idg_batch_set_schedule(p9idg_batch *batch, int32_t schedule);
p9idg_status p9idg_batch_synchronize(p9idg_batch *batch);
/* Per problem: ms from the start of the last degrid phase to the problem's last visibility (-1 if none). */
p9idg_status p9idg_batch_latencies(p9idg_batch *batch, double *ms);
p9idg_status p9idg_batch_get_stream(const p9idg_batch *batch, void **cuda_stream);
void p9idg_batch_destroy(p9idg_batch *batch);

/* Autotuner: times grid + degrid on a sample of the observation's baselines for each candidate
 * subgrid size (and work-item size) and returns the fastest per gridded visibility among the
 * candidates that grid at least 99.9 % of the best candidate's gridded visibilities.
 * subgrid_sizes NULL (or nsizes 0): 24, 32 and 48; a size the mode does not run (48 in a
 * tensor-core mode) or a plan it rules out is skipped. */
typedef struct p9idg_tuning {
    int32_t subgrid_size;
    int32_t kernel_size;
    int32_t gridder_max_vis;
    int32_t degridder_max_vis;
    double seconds_per_gridded_vis;  /* grid + degrid, measured on the sample */
    double gridded_fraction;         /* of the sample's visibilities */
} p9idg_tuning;
p9idg_status p9idg_autotune(const p9idg_params *c, const double *uvw, int32_t nbl, int32_t nt,
                            const double *frequencies, int32_t nch, int32_t mode, const int32_t *subgrid_sizes,
                            int32_t nsizes, p9idg_tuning *out);

/* ---------------- deconvolution side of the serial major cycle ---------------- */

/* FastSerialCD (Core/Deconvolution/FastSerialCD.cs), the IDeconvolver of the serial major cycle,
 * on the GPU with the reference's float arithmetic: the same pixel sequence, values and
 * iteration count.  Created like `new FastSerialCD(totalSize, psf)` (FastSerialCD.cs:31-46):
 * total size n x n, square PSF; PSF^2 (PSF.CalcPSFSquared) and the Lipschitz map
 * (PSF.CalcAMap) are built on the device. */
typedef struct p9idg_cd p9idg_cd;
/* DeconvolutionResult (IDeconvolver.cs:9-21). */
typedef struct p9idg_cd_result {
    int32_t converged;
    int32_t iterations;
    double elapsed_ms;
} p9idg_cd_result;
p9idg_status p9idg_cd_create(int32_t n, const float *psf, int32_t psf_h, int32_t psf_w, p9idg_cd **out);
/* FastSerialCD.MaxLipschitz (max of PSF^2). */
p9idg_status p9idg_cd_max_lipschitz(const p9idg_cd *cd, float *out);
/* Copies of the device PSF^2 ([2 psf_h][2 psf_w]) and Lipschitz map ([n][n]); either may be NULL. */
p9idg_status p9idg_cd_get_maps(p9idg_cd *cd, float *psf2_out, float *amap_out);
p9idg_status p9idg_cd_psf2_size(const p9idg_cd *cd, int32_t *h, int32_t *w);
/* Stream for the calls below (NULL = the deconvolver's own). */
p9idg_status p9idg_cd_set_stream(p9idg_cd *cd, void *cuda_stream);
/* FastSerialCD.Deconvolve (FastSerialCD.cs:76-102, 111-114): x (reconstruction) and bmap
 * (gradients) float[n][n] are updated in place, as the reference does.  P9IDG_INVALID_ARGUMENT
 * where the reference would index pixel (-1, -1) (epsilon <= 0 and no pixel changes). */
p9idg_status p9idg_cd_deconvolve(p9idg_cd *cd, float *x, float *bmap, float lambda, float alpha, int32_t max_iter,
                                 float epsilon, p9idg_cd_result *result);
p9idg_status p9idg_cd_deconvolve_device(p9idg_cd *cd, float *d_x, float *d_bmap, float lambda, float alpha,
                                        int32_t max_iter, float epsilon, p9idg_cd_result *result);
/* FastSerialCD.DeconvolvePath (FastSerialCD.cs:49-74, 106-109). */
p9idg_status p9idg_cd_deconvolve_path(p9idg_cd *cd, float *x, float *bmap, float lambda_min, float lambda_factor,
                                      float alpha, int32_t max_path_iter, int32_t max_iter, float epsilon,
                                      p9idg_cd_result *result);
/* FastSerialCD.GetAbsMaxDiff (FastSerialCD.cs:129-132). */
p9idg_status p9idg_cd_get_abs_max_diff(p9idg_cd *cd, const float *x, const float *bmap, float lambda, float alpha,
                                       float *out);
p9idg_status p9idg_cd_get_abs_max_diff_device(p9idg_cd *cd, const float *d_x, const float *d_bmap, float lambda,
                                              float alpha, float *out);
/* FastSerialCD.ResetLipschitzMap (FastSerialCD.cs:116-127), square PSF. */
p9idg_status p9idg_cd_reset_lipschitz_map(p9idg_cd *cd, const float *psf, int32_t h, int32_t w);
void p9idg_cd_destroy(p9idg_cd *cd);

/* PaddedConvolver (Core/PaddedConvolver.cs) in FP64 on the device.  _create takes the Fourier
 * kernel as `new PaddedConvolver(Complex[,] kernel, Rectangle kernelSize)` does (:36-41);
 * _create_correlation builds it from a PSF on the device, = new PaddedConvolver(
 * PSF.CalcPaddedFourierCorrelation(psf, (0, 0, n, n)), psf rectangle) (MajorCycle.cs:73). */
typedef struct p9idg_convolver p9idg_convolver;
p9idg_status p9idg_convolver_create(const double *kernel, int32_t h, int32_t w, int32_t kernel_h, int32_t kernel_w,
                                    p9idg_convolver **out);
p9idg_status p9idg_convolver_create_correlation(const float *psf, int32_t psf_h, int32_t psf_w, int32_t n,
                                                p9idg_convolver **out);
/* PaddedConvolver.Convolve (PaddedConvolver.cs:43-65): image float[n][n] -> out float[n][n]. */
p9idg_status p9idg_convolver_convolve(p9idg_convolver *conv, const float *image, int32_t n, float *out);
p9idg_status p9idg_convolver_convolve_device(p9idg_convolver *conv, const float *d_image, int32_t n, float *d_out);
void p9idg_convolver_destroy(p9idg_convolver *conv);

/* PSF helpers (Core/Common.cs) computed on the device.
 * CalcPaddedFourierCorrelation (:123-139): out complex[pad_y + h][pad_x + w] (must be square).
 * CalcPSFSquared (:162-174): out float[2h][2w].  CalcAMap(psf, (0, 0, total_h, total_w)) (:76-105). */
p9idg_status p9idg_psf_padded_fourier_correlation(const float *psf, int32_t h, int32_t w, int32_t pad_y,
                                                  int32_t pad_x, double *out);
p9idg_status p9idg_psf_squared(const float *psf, int32_t h, int32_t w, float *out);
p9idg_status p9idg_psf_amap(const float *psf, int32_t h, int32_t w, int32_t total_h, int32_t total_w, float *out);

/* MajorCycle.ReconstructSerialCD (SingleReconstruction/MajorCycle.cs:33-134) with the plan's
 * gridder (its precision mode), FastSerialCD and the padded correlation, all on the device;
 * the FITS writes of the reference are left out. */
typedef struct p9idg_mc_params {
    int32_t psf_cut_factor;     /* psfCutFactor */
    int32_t max_major_cycles;   /* maxMajorCycle */
    int32_t deconv_iterations;  /* deconvIterations */
    int32_t reserved;
    float lambda, alpha;
    float deconv_epsilon;       /* deconvEpsilon */
    float major_epsilon;        /* MAJOR_EPSILON, 1e-4f in the reference (MajorCycle.cs:18) */
} p9idg_mc_params;
/* What one major cycle computed, and its device time per phase. */
typedef struct p9idg_mc_cycle {
    float max_dirty, max_b, current_lambda, abs_max;
    int32_t deconvolved, converged, iterations, reserved;
    double grid_ms;    /* IDG.GridW of the residual visibilities */
    double image_ms;   /* WStackIFFTFloat + Shift + the gradient correlation */
    double deconv_ms;  /* GetAbsMaxDiff + Deconvolve */
    double degrid_ms;  /* model FFT + IDG.DeGridW + Visibilities.Substract */
    double objective;  /* Residuals.CalcPenalty(dirty) + ElasticNet.CalcPenalty(x, lambdaTrue, alpha) before
                          this cycle's deconvolution (MajorCycle.cs:102) */
} p9idg_mc_cycle;
/* Host arrays: vis complex128[nbl][nt][nch] (data.Visibilities), flags 1 byte per sample;
 * model_out (xImage) and residual_out (the last cycle's dirty image) float[N][N]; psf_out may be
 * NULL; cycles[max_major_cycles]; *ncycles = cycles run. */
p9idg_status p9idg_major_cycle_serial_cd(p9idg_plan *plan, const p9idg_mc_params *params, const double *vis,
                                         const uint8_t *flags, float *model_out, float *residual_out, float *psf_out,
                                         p9idg_mc_cycle *cycles, int32_t *ncycles);
/* Device buffers: d_vis complex64, d_flags uint8, d_model / d_residual / d_psf (may be NULL) float[N][N]. */
p9idg_status p9idg_major_cycle_serial_cd_device(p9idg_plan *plan, const p9idg_mc_params *params, const void *d_vis,
                                                const uint8_t *d_flags, float *d_model, float *d_residual,
                                                float *d_psf, p9idg_mc_cycle *cycles, int32_t *ncycles);

/* ---------------- FITS input/output of the reference's data layout (Core/FitsIO.cs) ---------------- */
/* Host-side, no GPU needed.  Primary-HDU arrays, big-endian; shapes are FITS axes (NAXIS1 first). */
p9idg_status p9idg_fits_shape(const char *path, int32_t *bitpix, int32_t *naxis, int64_t *axes, int32_t max_axes);
/* FitsIO.ReadUVW(file, fromBl, toBl) (FitsIO.cs:196-242): out double[to-from][nt][3], v negated. */
p9idg_status p9idg_fits_read_uvw(const char *path, int32_t from_bl, int32_t to_bl, double *out);
/* FitsIO.ReadFrequencies (FitsIO.cs:186-191). */
p9idg_status p9idg_fits_read_frequencies(const char *path, double *out, int64_t capacity);
/* FitsIO.ReadVisibilities(file, fromBl, toBl, nt, nch, norm) (FitsIO.cs:262-326): out complex128
 * [to-from][nt][nch] = (XX + YY) / norm, from polarisations 0 and 3. */
p9idg_status p9idg_fits_read_visibilities(const char *path, int32_t from_bl, int32_t to_bl, int32_t nt, int32_t nch,
                                          double norm, double *out);
/* FitsIO.ReadFlags(file, fromBl, toBl, nt, nch) (FitsIO.cs:328-389): out 1 byte each, 1 where the
 * polarisation values sum to non-zero. */
p9idg_status p9idg_fits_read_flags(const char *path, int32_t from_bl, int32_t to_bl, int32_t nt, int32_t nch,
                                   uint8_t *out);
/* FitsIO.ReadImage (bitpix -32, float) / ReadImageDouble (-64, double) (FitsIO.cs:140-185). */
p9idg_status p9idg_fits_read_image(const char *path, int32_t bitpix, void *out, int64_t capacity);
/* FitsIO.Write<T>(T[,] img) (FitsIO.cs:64-84), float (-32) or double (-64) [rows][cols]. */
p9idg_status p9idg_fits_write_image(const char *path, int32_t bitpix, const void *data, int32_t rows, int32_t cols);

/* ---------------- stage timing (CUDA events on the plan's stream) ---------------- */

enum {
    P9IDG_STAGE_GRIDDER = 0,
    P9IDG_STAGE_SUBGRID_IFFT_ADD = 1,
    P9IDG_STAGE_SPLIT_SUBGRID_FFT = 2,
    P9IDG_STAGE_DEGRIDDER = 3,
    P9IDG_STAGE_LAYER_FFT = 4,
    P9IDG_STAGE_H2D = 5,
    P9IDG_STAGE_D2H = 6,
    P9IDG_STAGE_CONVERT = 7,
    P9IDG_NUM_STAGES = 8
};

p9idg_status p9idg_plan_enable_timing(p9idg_plan *plan, int32_t on);
/* Accumulated milliseconds and launch counts per stage since the last reset (synchronises). */
p9idg_status p9idg_plan_stage_times(p9idg_plan *plan, double *ms, int64_t *launches);
p9idg_status p9idg_plan_reset_timing(p9idg_plan *plan);

/* ---------------- misc ---------------- */

const char *p9idg_last_error(void);
const char *p9idg_version(void);
/* Number of visible CUDA devices (0 when none); does not create a context. */
int32_t p9idg_device_count(void);
/* Measured FP32 sincos throughput of the current device (sincos per second) from a short
 * on-device loop of the intrinsic the FP32 kernels use; the FP32/SFU roofline denominator. */
p9idg_status p9idg_measure_sincos_peak(double *sincos_per_s, double *fma_per_s);
/* Runs a known 128 x n x 64 GEMM (n = 32, 64 or 128) through the tensor-core operand layout,
 * descriptors and TMEM path the P9IDG_MODE_TC_* kernels use; *max_rel_err is the largest error
 * relative to max |C| (inputs are exactly representable, so it is at FP32-accumulation level). */
p9idg_status p9idg_tc_selftest(int32_t mode, int32_t n, double *max_rel_err);
/* Fault injection for callers' error-path tests (no counterpart in the reference): after
 * `after` more successful device allocations, every device allocation the library makes for its
 * plans, deconvolvers and tensor-core state fails as cudaMalloc does when memory runs out, so the
 * calls return P9IDG_OUT_OF_MEMORY; after < 0 turns it off.  Process-wide. */
p9idg_status p9idg_debug_fail_device_allocations(int64_t after);
/* Fault injection for the tensor-core kernels' bounded waits (no counterpart in the reference):
 * later single-plan launches wait at most wait_ns per pipeline wait (0 = the default 2 s) and, if
 * skip_stage >= 0, their loader warp never delivers input stage skip_stage of a work item, so the
 * waits for it run out: the kernel frees its tensor memory once its issued MMAs have finished
 * and the call returns P9IDG_DEVICE_CHECK_FAILED.  (0, -1) restores normal operation.  Process-wide. */
p9idg_status p9idg_debug_tc_wait(int64_t wait_ns, int32_t skip_stage);

#ifdef __cplusplus
}
#endif

#endif /* P9IDG_H */
