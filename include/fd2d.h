/*
 * fd2d.h -- C ABI of the GB300 fd2d_noise wave-propagation library (libfd2d.so).
 *
 * The three solver entry points replace the MATLAB solvers of fd2d_noise,
 * which its callers reach under the MATLAB-Coder names run_*_mex:
 *
 *   fd2d_forward1_green        <- code/run_forward1_green.m:1
 *   fd2d_forward2_correlation  <- code/run_forward2_correlation.m:1
 *   fd2d_noise_adjoint         <- code/run_noise_adjoint.m:1
 *
 * Argument order and meaning follow the MATLAB signatures and the codegen type
 * specification in code/mex_functions/compile_all.m:5-34.  The MATLAB solvers
 * read their configuration from input_parameters(), input_interferometry() and
 * absorb_specs() (input/input_parameters.m:2-88, input/input_interferometry.m:2-21,
 * input/absorb_specs.m:2-15); here that configuration travels explicitly in
 * fd2d_config.
 *
 * Conventions
 *  - Arrays are column-major with x fastest, exactly as MATLAB stores them:
 *    element (ix, iz, k) of an nx-by-nz-by-K array is at ix + nx*(iz + nz*k)
 *    (0-based).  A 2-D n-by-m array (src, rec, spectrum, seismograms) has
 *    element (i, j) at i + n*j.
 *  - Complex arrays are split into separate real and imaginary planes (the
 *    non-interleaved MEX convention).
 *  - A NULL pointer (with count 0) stands for the MATLAB empty array [] /
 *    single([]) / complex([]).
 *  - Outputs are caller-allocated; fd2d_query_sizes() gives their sizes.  The
 *    library never frees caller memory.
 *  - By default every pointer is a HOST pointer and a call is synchronous.
 *    After fd2d_ctx_set_memspace(ctx, FD2D_MEM_DEVICE) every array pointer is a
 *    device pointer of the context's GPU and the call is asynchronous on the
 *    context's stream (scalars and fd2d_config.f_sample stay on the host).
 *  - Errors are returned as fd2d_status; fd2d_last_error() gives the message.
 *    The library never exits or aborts.
 */
#ifndef FD2D_H
#define FD2D_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define FD2D_ABI_VERSION 1

typedef enum fd2d_status {
  FD2D_OK = 0,
  FD2D_ERR_ARG = 1,       /* NULL where an array is required, bad scalar      */
  FD2D_ERR_SHAPE = 2,     /* array sizes inconsistent with the configuration   */
  FD2D_ERR_ORDER = 3,     /* finite-difference order not in {2, 4, 6, 8}       */
  FD2D_ERR_OOM = 4,       /* device memory exhausted                           */
  FD2D_ERR_CUDA = 5,      /* CUDA runtime or launch error                      */
  FD2D_ERR_TIMEOUT = 6,   /* a bounded device-side wait gave up                */
  FD2D_ERR_INDEX = 7,     /* the MATLAB solver would index out of range here   */
  FD2D_ERR_NO_DEVICE = 8, /* no usable CUDA device                             */
  FD2D_ERR_UNSUPPORTED = 9
} fd2d_status;

typedef enum fd2d_precision {
  FD2D_PREC_FP64 = 0, /* plain FP64 form: the reference arithmetic on the GPU  */
  FD2D_PREC_FP32 = 1  /* FP32 stencil + split-TF32 tensor-core contractions     */
} fd2d_precision;

typedef enum fd2d_memspace { FD2D_MEM_HOST = 0, FD2D_MEM_DEVICE = 1 } fd2d_memspace;

/* Hidden inputs of the MATLAB solvers, made explicit. */
typedef struct fd2d_config {
  /* input_parameters() -- input/input_parameters.m:2-88 */
  double Lx, Lz;          /* domain extent [m]                                  */
  int32_t nx, nz;         /* grid points                                        */
  double dt;              /* time step [s]                                      */
  int32_t nt;             /* forward time steps                                 */
  int32_t order;          /* FD order: 2 and 4 as in the reference; 6 and 8 are
                             the staggered-grid extension (no reference analogue) */
  int32_t n_basis_fct;    /* frequency bands of the source model (0 = none)     */
  int32_t fw_nth;         /* store every fw_nth step of the forward field       */
  /* input_interferometry() -- input/input_interferometry.m:16-21 */
  int32_t n_sample;       /* number of frequencies                              */
  const double* f_sample; /* n_sample frequencies [Hz], evenly spaced (host)    */
  int32_t freq_samp;      /* DFT / injection decimation                         */
  /* absorb_specs() -- input/absorb_specs.m:8-15 */
  double absorb_width;    /* taper width [m]                                    */
  int32_t absorb_left, absorb_right, absorb_top, absorb_bottom;
} fd2d_config;

/* Output sizes (in elements) for a configuration and receiver count. */
typedef struct fd2d_sizes {
  int32_t ntc;            /* 2*nt-1: correlation / adjoint time steps          */
  int32_t n_fw_green;     /* G_out planes (code/run_forward1_green.m:98-103)   */
  int32_t n_fw_corr;      /* C_out / u_out planes: floor(ntc/fw_nth)           */
  int32_t n_kernel_planes;/* K planes: n_basis_fct+1, or 2 when n_basis_fct==0 */
  int64_t npts;           /* nx*nz                                             */
  int64_t G_fft;          /* nx*nz*n_sample (per real/imag plane set)          */
  int64_t G_out;          /* nx*nz*n_fw_green                                  */
  int64_t seis_green;     /* nr*nt                                             */
  int64_t C_out;          /* nx*nz*n_fw_corr                                   */
  int64_t seis_corr;      /* nr*ntc                                            */
  int64_t K;              /* nx*nz*n_kernel_planes                             */
} fd2d_sizes;

typedef struct fd2d_ctx fd2d_ctx;

/* ---- context --------------------------------------------------------------- */
int32_t fd2d_abi_version(void);
/* Create a context on CUDA device `device` computing in `precision`. */
fd2d_status fd2d_ctx_create(int32_t device, int32_t precision, fd2d_ctx** out);
fd2d_status fd2d_ctx_destroy(fd2d_ctx* ctx);
/* Use `stream` (a cudaStream_t) for all work of this context; NULL = own stream. */
fd2d_status fd2d_ctx_set_stream(fd2d_ctx* ctx, void* stream);
fd2d_status fd2d_ctx_set_memspace(fd2d_ctx* ctx, int32_t memspace);
fd2d_status fd2d_ctx_set_precision(fd2d_ctx* ctx, int32_t precision);
/* Wait for all work queued on the context's stream. */
fd2d_status fd2d_ctx_synchronize(fd2d_ctx* ctx);
/* Device-memory bounds of the FP32 form: at most `max_snapshots` stored
 * snapshots per DFT contraction (rounded down to a multiple of 32; 0 = 640)
 * and `max_injection_planes` resident injection planes (rounded down to a
 * multiple of 128; 0 = as many as fit in 4 GiB).  Smaller chunks use less
 * memory at the cost of more, smaller contractions.  Each DFT chunk is summed
 * in two FP32 halves and the chunks in FP64: longer chunks lose FP32 accuracy
 * (the default keeps FP32 mu kernels within 1e-4 of FP64 at nt 2500). */
fd2d_status fd2d_ctx_set_chunks(fd2d_ctx* ctx, int32_t max_snapshots, int32_t max_injection_planes);
/* Tile rows of the FP32 step kernel (tiles are 32 points wide): 16, 30, 32 or
 * 40 to force a shape; FD2D_TILE_ROWS_AUTO (0, default) to time every shape once
 * per context for each grid, FD order and lane count when the stream is idle
 * and keep the fastest (the size rule otherwise); FD2D_TILE_ROWS_RULE (-1) for
 * the size rule only (fewest waves of resident CTAs, the shortest tiles among
 * equals).  The environment variable FD2D_TILE_ROWS forces a shape for
 * contexts left at 0. */
#define FD2D_TILE_ROWS_AUTO 0
#define FD2D_TILE_ROWS_RULE (-1)
fd2d_status fd2d_ctx_set_tile_rows(fd2d_ctx* ctx, int32_t rows);
/* Tile rows used by the last FP32 time loop this context set up (0: none yet). */
int32_t fd2d_ctx_last_tile_rows(const fd2d_ctx* ctx);
/* Time steps per launch of the FP32 time loops at FD orders 2 and 4: 1 or 2
 * to force, 0 (default) to time both, with every tile shape, once per context
 * for each grid, order, lane count and kind when the stream is idle and keep
 * the fastest (one step per launch otherwise).  Two steps per launch
 * recompute the first step on a wider halo ring -- more arithmetic for half
 * the launches, which pays where a launch leaves most SMs idle (small grids);
 * the fields, seismograms, spectra and kernels are bit for bit those of one
 * step per launch.  The Green-function, correlation and adjoint loops pair
 * steps (stored wavefields are taken inside a pair); steps with something in
 * between (a K_mu term, a DFT or injection chunk boundary) run singly, and
 * Born runs, order 6/8 and the multi-geometry batch run one step per launch.  The environment variable
 * FD2D_TIME_DEPTH forces a depth for contexts left at 0. */
fd2d_status fd2d_ctx_set_time_depth(fd2d_ctx* ctx, int32_t depth);
/* Diagnostic of the bounded device-side waits: runs a kernel whose mbarrier
 * wait nothing completes, bounded by limit_us (1 .. 2e6) microseconds of
 * %globaltimer -- the wait every kernel of the library uses, there with a
 * 2 s limit.  It gives up, flags the context, and the call returns
 * FD2D_ERR_TIMEOUT after about limit_us; the context stays usable. */
fd2d_status fd2d_check_bounded_wait(fd2d_ctx* ctx, int64_t limit_us);
/* Steps per launch chosen for the last FP32 time loop this context set up (0: none yet). */
int32_t fd2d_ctx_last_time_depth(const fd2d_ctx* ctx);
/* Declare that other work (other contexts, processes or streams) runs on the
 * GPU beside this context's solves (1) or not (0, default).  Shared: time steps
 * are launched without programmatic early launch (a waiting step would hold
 * SM slots the other work could use) and tile shapes follow the size rule
 * (no timed trials).  Lane groups of one fd2d_correlation_batch call are
 * treated as shared among themselves automatically. */
fd2d_status fd2d_ctx_set_shared_gpu(fd2d_ctx* ctx, int32_t shared);
/* Device memory the context keeps between calls (workspace buffers). */
int64_t fd2d_ctx_workspace_bytes(const fd2d_ctx* ctx);
/* Wait for the stream, then free the workspace and the cached CUDA graphs;
 * *bytes (may be NULL) receives the workspace size that was freed.  Freed
 * workspace stays in the device's stream-ordered memory pool for reuse. */
fd2d_status fd2d_ctx_release(fd2d_ctx* ctx, int64_t* bytes);
/* Device memory the library can still allocate on `device`: the free bytes of
 * cudaMemGetInfo plus what the device's stream-ordered pool holds unused
 * (released workspace).  No reference counterpart: admission control of the
 * serving loop sizes its budget with it. */
fd2d_status fd2d_device_free_bytes(int32_t device, int64_t* free_bytes, int64_t* total_bytes);
/* Kernels launched by this context since creation (instrumentation). */
int64_t fd2d_ctx_kernel_launches(const fd2d_ctx* ctx);
/* Device-time instrumentation.  When enabled, every launch of the classes
 * below is bracketed by CUDA events on the context's stream; fd2d_ctx_timing()
 * waits for the stream, returns per class the summed milliseconds, the launch
 * count and the work units (grid-point updates for stencils, multiply-adds for
 * contractions), then resets the counters. */
enum {
  FD2D_TIMER_STEP_V = 0,   /* stencil step without displacement (Green run)  */
  FD2D_TIMER_STEP_VU = 1,  /* stencil step with u (correlation / adjoint)    */
  FD2D_TIMER_CONTRACT = 2, /* DFT / injection contractions, operand images    */
  FD2D_TIMER_COUNT = 3
};
fd2d_status fd2d_ctx_set_timing(fd2d_ctx* ctx, int32_t enable);
fd2d_status fd2d_ctx_timing(fd2d_ctx* ctx, double* ms, int64_t* launches, int64_t* units);
/* Message of the last error on this context ("" if none). ctx may be NULL for
   errors raised before a context existed. */
const char* fd2d_last_error(const fd2d_ctx* ctx);

/* Validate a configuration and compute output sizes (no GPU needed). */
fd2d_status fd2d_query_sizes(const fd2d_config* cfg, int32_t nr, fd2d_sizes* out);

/* ---- solvers ----------------------------------------------------------------
 * [G_fft, G_out, seismograms] = run_forward1_green(mu, rho, src, rec, mode, dmu, G_in)
 * code/run_forward1_green.m:1-201.
 *   mu, rho      nx*nz
 *   src          ns-by-2 (x, z) [m]      rec   nr-by-2
 *   mode         0: no wavefield output; otherwise G_out is stored
 *   dmu          nx*nz or NULL; when given the run is the Born (dG) run driven
 *                by dt*dmu*grad(G_in) and the point source is off
 *   G_in         nx*nz*n_G_in single, needs n_G_in >= nt when dmu is given
 *   G_fft_re/im  out, nx*nz*n_sample, returned conjugated as the reference does
 *   G_out        out, nx*nz*n_fw_green single (only written when mode != 0)
 *   seismograms  out, nr*nt (velocity at the receivers)                       */
fd2d_status fd2d_forward1_green(fd2d_ctx* ctx, const fd2d_config* cfg,
                                const double* mu, const double* rho,
                                const double* src, int32_t ns,
                                const double* rec, int32_t nr,
                                int32_t mode,
                                const double* dmu,
                                const float* G_in, int32_t n_G_in,
                                double* G_fft_re, double* G_fft_im,
                                float* G_out,
                                double* seismograms);

/* [seismograms, C_out] = run_forward2_correlation(mu, rho, G_fft, spectrum,
 *                                   source_dist, rec, mode, dmu, C_in)
 * code/run_forward2_correlation.m:1-254.
 *   G_fft_re/im  nx*nz*n_G (n_G >= n_sample): conjugated Green spectrum
 *   spectrum     n_sample-by-n_noise_sources
 *   source_dist  nx*nz*n_dist: n_dist == n_noise_sources when n_basis_fct == 0
 *                (the reference only runs with one), n_dist == n_basis_fct
 *                otherwise
 *   dmu, C_in    Born term -dmu*grad(C_in(n) - C_in(n+1)); C_in needs ntc planes
 *   seismograms  out, nr*ntc: displacement at the receivers = the correlations
 *   C_out        out, nx*nz*n_fw_corr single (only written when mode != 0)    */
fd2d_status fd2d_forward2_correlation(fd2d_ctx* ctx, const fd2d_config* cfg,
                                      const double* mu, const double* rho,
                                      const double* G_fft_re, const double* G_fft_im,
                                      int32_t n_G,
                                      const double* spectrum, int32_t n_noise_sources,
                                      const double* source_dist, int32_t n_dist,
                                      const double* rec, int32_t nr,
                                      int32_t mode,
                                      const double* dmu,
                                      const float* C_in, int32_t n_C_in,
                                      double* seismograms,
                                      float* C_out);

/* [K, stf_fft, u_out, seismograms] = run_noise_adjoint(mu, rho, u_fwd, stf, src,
 *                 rec, spectrum, source_dist, G_fft, mode, dmu, u_in)
 * code/run_noise_adjoint.m:1-368.
 *   u_fwd        nx*nz*n_u_fwd single forward snapshots (NULL = none: no K_mu)
 *   stf_re/im    stf_dims = {d0, d1, d2}.  d2 == 1: point adjoint sources,
 *                d0 >= ns rows by d1 >= ntc columns (only the real part is used).
 *                d2 > 1: field source, nx*nz*d2 with d2 >= n_sample.
 *                NULL / d0*d1*d2 == 0: no source.
 *   src          ns-by-2 adjoint source positions
 *   spectrum     n_sample-by-n_noise_sources (NULL if unused)
 *   source_dist  nx*nz*n_dist (NULL: no field source)
 *   G_fft_re/im  nx*nz*n_G; the source kernel is built when n_G == n_sample
 *   mode         0, 1, 10, 11, 12, 13 as in code/run_noise_adjoint.m:17-22
 *   dmu, u_in    Born term; active when u_in has exactly ntc planes
 *   K            out, nx*nz*n_kernel_planes: source kernel planes then K_mu
 *   stf_fft_re/im out, nx*nz*n_sample (written for modes 1, 12, 13; zero else)
 *   u_out        out, nx*nz*n_fw_corr single (modes 11 and 13)
 *   seismograms  out, nr*ntc                                                   */
fd2d_status fd2d_noise_adjoint(fd2d_ctx* ctx, const fd2d_config* cfg,
                               const double* mu, const double* rho,
                               const float* u_fwd, int32_t n_u_fwd,
                               const double* stf_re, const double* stf_im,
                               const int64_t stf_dims[3],
                               const double* src, int32_t ns,
                               const double* rec, int32_t nr,
                               const double* spectrum, int32_t n_noise_sources,
                               const double* source_dist, int32_t n_dist,
                               const double* G_fft_re, const double* G_fft_im,
                               int32_t n_G,
                               int32_t mode,
                               const double* dmu,
                               const float* u_in, int32_t n_u_in,
                               double* K,
                               double* stf_fft_re, double* stf_fft_im,
                               float* u_out,
                               double* seismograms);

/* ---- batches -------------------------------------------------------------------
 * One job is one reference station of the parfor loop of
 * code/calculate_data.m:189-202: the Green function (run_forward1_green,
 * mode 0) followed by the correlation wavefield (run_forward2_correlation,
 * mode 0); the job returns the correlations.  Jobs may have different
 * configurations (grid sizes, nt) and models.  Arrays follow the context's
 * memspace.  In FP32 the jobs advance concurrently, in groups whose device
 * buffers fit in the memory budget (default: 80 % of the free device memory at
 * the call): jobs of one configuration and receiver count are lanes of the same
 * launches (one stencil launch per time step for all of them, one DFT and one
 * injection contraction over all their grid points), and jobs of different
 * configurations run as parallel branches of one CUDA graph.
 * In FP64 (the plain form) the jobs run one after another. */
typedef struct fd2d_job {
  const fd2d_config* cfg;
  const double* mu;
  const double* rho;
  const double* spectrum;     /* n_sample-by-n_noise_sources */
  int32_t n_noise_sources;
  const double* source_dist;  /* nx*nz*n_dist */
  int32_t n_dist;
  const double* src;          /* 1-by-2 reference station [m] */
  const double* rec;          /* nr-by-2 receivers [m] */
  int32_t nr;
  double* correlations;       /* out: nr*(2*nt-1) */
} fd2d_job;
fd2d_status fd2d_correlation_batch(fd2d_ctx* ctx, const fd2d_job* jobs, int32_t n_jobs);
/* Device-memory budget of a batch in bytes (0 = 80 % of the free memory). */
fd2d_status fd2d_ctx_set_memory_budget(fd2d_ctx* ctx, int64_t bytes);
/* Launch groups of the last batch on ctx: writes up to `cap` lane counts (jobs
 * advanced by one launch per step, in execution order) and returns the number
 * of groups. */
int32_t fd2d_ctx_last_batch(const fd2d_ctx* ctx, int32_t* lanes, int32_t cap);

/* ---- measurements ---------------------------------------------------------------
 * [misfit_n, adstf] = make_adjoint_sources(u, u_0, du, t, veldis, measurement,
 *                                          src, rec, deriv_order)
 * tools/measurement/make_adjoint_sources.m:31-175 with log_amp_ratio.m:23-93
 * (fixed 100-200 s Hann window on the causal branch and its mirror, :87-103),
 * waveform_difference.m:23-48 (cos-taper window over the whole axis),
 * cc_time_shift.m:21-61 and amp_diff.m:22-66 (cos-taper windows over
 * 100-200 s and -200 to -100 s, misfits and adjoint sources summed), FP64.
 *   measurement   FD2D_MEAS_*
 *   deriv_order   1 ('1st': misfit and adjoint source) or 2 ('2nd': the
 *                 Hessian adjoint source along du; misfit_n is set to 0)
 *   velocity      0 'dis', 1 'vel' (u, u_0 differentiated; adstf corrected)
 *   u, u_0, du    n_rec-by-nt (du only for deriv_order 2)
 *   t             nt time samples, HOST pointer (dt = |t(2) - t(1)|)
 *   misfit        out, n_rec (may be NULL)        adstf  out, n_rec-by-nt
 * The source/receiver positions of the MATLAB signature only feed commented-out
 * window choices there and are not arguments.  nt <= 20480. */
enum {
  FD2D_MEAS_WAVEFORM_DIFFERENCE = 0,  /* tools/measurement/waveform_difference.m */
  FD2D_MEAS_LOG_AMPLITUDE_RATIO = 1,  /* tools/measurement/log_amp_ratio.m */
  FD2D_MEAS_CC_TIME_SHIFT = 2,        /* tools/measurement/cc_time_shift.m (first order only) */
  FD2D_MEAS_AMPLITUDE_DIFFERENCE = 3  /* tools/measurement/amp_diff.m */
};
fd2d_status fd2d_make_adjoint_sources(fd2d_ctx* ctx, int32_t measurement, int32_t deriv_order, int32_t velocity,
                                      const double* u, const double* u_0, const double* du, int32_t n_rec,
                                      int32_t nt, const double* t, double* misfit, double* adstf);

/* ---- model maps -----------------------------------------------------------------
 * GY = gaussblur2d(Y, x1, x2, sigma) -- tools/addons/gaussblur2d.m:2-38, FP64:
 * Gaussian weights exp(-(d/sigma)^2/2) within sqrt(14)*sigma along each axis,
 * normalised by the weight sums.  Y and GY are n1-by-n2; x1 (n1) and x2 (n2)
 * the coordinates.  Arrays follow the context's memspace. */
fd2d_status fd2d_gaussblur2d(fd2d_ctx* ctx, const double* Y, int32_t n1, int32_t n2, const double* x1,
                             const double* x2, double sigma1, double sigma2, double* GY);

/* B = imfilter(Y, h, 'circular') -- the structure-plane smoothing of the 'ring'
 * parameterisation (inversion/optlib_callback_fct/map_m_to_parameters.m:28,
 * map_gradparameters_to_gradm.m:34), FP64: correlation with the m1-by-m2
 * kernel h, output n1-by-n2 like Y, Y extended periodically, the centre of h at
 * floor((size(h)+1)/2) (1-based).  Arrays are column-major and follow the
 * context's memspace. */
fd2d_status fd2d_imfilter_circular(fd2d_ctx* ctx, const double* Y, int32_t n1, int32_t n2, const double* h,
                                   int32_t m1, int32_t m2, double* B);

/* ---- building block ----------------------------------------------------------
 * R[n*ldr + m] = sum_{k<Kd} A[k*lda + m] * B[k*ldb + n]  for m < M, n < N:
 * the split-TF32 tensor-core contraction behind the on-the-fly DFT
 * (code/run_forward1_green.m:176-183) and the correlation-source injection
 * (code/run_forward2_correlation.m:195-216).  Device pointers, FP32, queued on
 * the context's stream.  No reference counterpart as a separate function. */
fd2d_status fd2d_contract_f32(fd2d_ctx* ctx, const float* A, int64_t lda, const float* B, int64_t ldb,
                              int32_t M, int32_t N, int32_t Kd, float* R, int64_t ldr);

/* ---- allocation-free Green-function seismograms --------------------------------
 * No counterpart in the reference: an extra entry point for callers that must
 * not allocate GPU memory -- hosts that own a fixed device-memory budget, or run
 * inside a runtime whose allocator they do not control, so that any cudaMalloc
 * could fail or stall mid-run.  It runs the FP32 Green-function time loop of
 * fd2d_forward1_green (mode 0, point force 1e9 at `src`) and returns only the
 * velocity seismograms; no spectra, no snapshots, no context.
 *   mu, rho, seismograms  DEVICE pointers (nx*nz, nx*nz, nr*nt doubles)
 *   src, rec              HOST pointers (ns-by-2, nr-by-2 positions [m])
 *   stream                cudaStream_t to queue the work on (NULL: default stream)
 * All working memory is one statically sized device array compiled into the
 * library (FD2D_NOALLOC_SCRATCH_BYTES per GPU, held until the process exits):
 * 9 FP32 planes of ((nx rounded up to 32) * nz) floats plus 8 bytes per source
 * and receiver must fit, else FD2D_ERR_SHAPE.  The first call on a device looks
 * up that array's device address (make that first call before any stream
 * capture).  Every call reuses the same array, so calls whose work overlaps on
 * the GPU (other streams, other host threads) race: serialise them.  The call
 * waits for its own work on `stream` before it returns (it reads the
 * device-side error flag back).  Its seismograms are bit-identical to those of
 * fd2d_forward1_green in FP32, mode 0, on the same inputs. */
#define FD2D_NOALLOC_SCRATCH_BYTES (16u << 20)
fd2d_status fd2d_forward1_seismograms_noalloc(const fd2d_config* cfg, const double* mu, const double* rho,
                                              const double* src, int32_t ns, const double* rec, int32_t nr,
                                              double* seismograms, void* stream);

#ifdef __cplusplus
}
#endif

#endif /* FD2D_H */
