/*
 * tealeaf_capi.h -- C-ABI of libtealeaf_gb300.so, the GB300 (sm_103a) CUDA
 * implementation of TeaLeaf's implicit heat-conduction solve.
 *
 * Two layers:
 *
 *  1. The reference's own entry points, same symbol names and by-reference
 *     arguments as the gfortran-mangled `*_kernel_cuda_` functions of
 *     UK-MAC/TeaLeaf_CUDA, so the unchanged Fortran wrappers (tea_leaf_cg.f90,
 *     tea_leaf_common.f90, tea_leaf_ppcg.f90, tea_leaf_cheby.f90,
 *     field_summary.f90, update_halo.f90, build_field.f90, generate_chunk.f90,
 *     initialise_chunk.f90, set_field.f90) link against this library in place
 *     of the reference's *_kernel_cuda.cu objects.  Each comment cites the
 *     reference definition it replaces.  They act on one process-wide chunk,
 *     created by initialise_cuda_, exactly like the reference's `cuda_chunk`
 *     singleton (init_cuda.cu:33).  They return nothing, as in the reference;
 *     an error is recorded and can be read with tl_last_error().
 *
 *  2. The `tl_*` API: explicit chunk handles, an explicit configuration
 *     struct instead of the reference's second scan of ./tea.in
 *     (init_cuda.cu:63-163), integer status codes, and a device-resident
 *     solve (tl_timestep) that keeps alpha/beta and the exit test on the GPU.
 *
 * All device memory is owned by the library; callers pass host scalars and
 * host arrays only.  Fields crossing the boundary use the reference layout:
 * (x_cells + 2*halo) columns by (y_cells + 2*halo) rows, x fastest, as
 * THARR2D of kernel_files/cuda_kernel_header.hpp:27-29.
 */
#ifndef TEALEAF_CAPI_H
#define TEALEAF_CAPI_H

#ifdef __cplusplus
extern "C" {
#endif

/* ---------------------------------------------------------------- status */
#define TL_OK                    0
#define TL_WARN_MAXITER          1  /* tl_max_iters reached before tl_eps   */
#define TL_ERR_ARG              -1  /* bad argument or configuration        */
#define TL_ERR_CUDA             -2  /* a CUDA runtime call failed           */
#define TL_ERR_ALLOC            -3  /* device or host allocation failed     */
#define TL_ERR_BREAKDOWN        -4  /* NaN/Inf in a Krylov scalar           */
#define TL_ERR_STATE            -5  /* call out of order (no chunk, ...)    */
#define TL_ERR_DECK             -6  /* tea.in could not be parsed           */
#define TL_ERR_EIGEN            -7  /* eigenvalue estimate failed           */

/* ------------------------------------------------------------ enumerations
 * values as the reference: data.f90:62-75, cuda_common.hpp:32-55 */
#define TL_SOLVER_JACOBI         1
#define TL_SOLVER_CG             2
#define TL_SOLVER_CHEBYSHEV      3
#define TL_SOLVER_PPCG           4
#define TL_PREC_NONE             1
#define TL_PREC_JAC_DIAG         2
#define TL_PREC_JAC_BLOCK        3
#define TL_COEF_CONDUCTIVITY     1
#define TL_COEF_RECIP_CONDUCTIVITY 2
#define TL_GEOM_RECTANGLE        1
#define TL_GEOM_CIRCLE           2
#define TL_GEOM_POINT            3
/* numerical form of the solve (no reference counterpart) */
#define TL_PRECISION_FP64        0  /* plain FP64: the drop-in               */
#define TL_PRECISION_MIXED       1  /* FP32 inner Krylov + FP64 refinement   */
/* start of the implicit solve (no reference counterpart; tl_warm_start) */
#define TL_WARM_NONE             0  /* u = u^n, the reference's start        */
#define TL_WARM_LEARNED          1  /* network + previous increment, Galerkin */
#define TL_WARM_PREV             2  /* previous increment, Galerkin          */
/* the inner product of the warm start's projection (tl_set_warm_start_options) */
#define TL_WARM_PROJ_ENERGY      0  /* minimise the energy (A-norm of the error) */
#define TL_WARM_PROJ_RESIDUAL    1  /* minimise the residual's 2-norm        */
/* field ids: FIELD_* of data.f90:44-50 plus solver work arrays */
#define TL_FIELD_DENSITY         1
#define TL_FIELD_ENERGY0         2
#define TL_FIELD_ENERGY1         3
#define TL_FIELD_U               4
#define TL_FIELD_P               5
#define TL_FIELD_SD              6
#define TL_FIELD_R               7
#define TL_FIELD_U0              8
#define TL_FIELD_W               9
#define TL_FIELD_Z              10
#define TL_FIELD_KX             11
#define TL_FIELD_KY             12
#define TL_FIELD_MI             13
#define TL_FIELD_CP             14
#define TL_FIELD_BFP            15
#define TL_FIELD_VOLUME         16
#define TL_FIELD_RTEMP          17
#define TL_FIELD_UTEMP          18
#define TL_FIELD_R_STORE        19

#define TL_MAX_STATES           64

typedef struct tl_state {
    int geometry;                 /* TL_GEOM_*                               */
    double density, energy;
    double xmin, xmax, ymin, ymax, radius;
} tl_state_t;

/* Everything tea.in sets (read_input.f90:38-327).  State extents are stored
 * after read_input.f90:320-327 shrinks states 2..N by a hundredth of a cell. */
typedef struct tl_config {
    int x_cells, y_cells;
    double xmin, xmax, ymin, ymax;
    double dtinit, end_time;
    int end_step, summary_frequency;
    int max_iters;                /* tl_max_iters                            */
    double eps;                   /* tl_eps                                  */
    int solver;                   /* TL_SOLVER_*                             */
    int precond;                  /* TL_PREC_*                               */
    int coefficient;              /* TL_COEF_*                               */
    int halo_depth;
    int reflective_boundary;
    int check_result;             /* tl_check_result                         */
    int ch_cg_presteps;           /* tl_ch_cg_presteps                       */
    double ch_cg_epslim;          /* tl_ch_cg_epslim                         */
    int ppcg_inner_steps;         /* tl_ppcg_inner_steps                     */
    int profiler_on, verbose, test_problem, cuda_device;
    int precision;                /* TL_PRECISION_* (tl_precision)           */
    double inner_eps;             /* mixed: inner FP32 relative tolerance    */
    int warm_start;               /* TL_WARM_* (tl_warm_start)               */
    int nstates;
    tl_state_t states[TL_MAX_STATES];
} tl_config_t;

/* outcome of one implicit solve (one call of tea_leaf(), tea_solve.f90:37) */
typedef struct tl_solve_info {
    int status;                   /* TL_OK, TL_WARN_MAXITER or an error      */
    int iterations;               /* "Iteration count" (tea_solve.f90:452)   */
    int ppcg_inner_iters;         /* "PPCG Iteration count" (:457)           */
    int switch_n;                 /* CG iteration of the Chebyshev/PPCG switch */
    int est_itc;                  /* Chebyshev iteration estimate            */
    int outer_iters;              /* mixed: FP64 refinement steps            */
    int inner_iters;              /* mixed: FP32 Krylov iterations in total  */
    double initial_residual;
    double error;                 /* final |error|                           */
    double error_ratio;           /* "Conduction error" (tea_solve.f90:446)  */
    double exact_error_ratio;     /* tl_check_result (tea_solve.f90:449)     */
    double eigmin, eigmax;
    double rx, ry;
    double seconds;               /* wall time of the solve on the host      */
    int warm_used;                /* warm start taken (1) or u = u^n (0)     */
    double warm_ratio;            /* its residual / the plain start's        */
    double warm_net_share;        /* learned: the network direction's share of
                                     the start's energy decrease (0 when it
                                     was not consulted)                      */
} tl_solve_info_t;

typedef struct tl_chunk tl_chunk_t;

/* ------------------------------------------------------------- tl_* API */

/* tea.in text -> config, with parse.f90 / read_input.f90 semantics */
int tl_parse_deck(const char *deck_text, tl_config_t *cfg, char *err, int errlen);
/* message of the most recent error on this thread ("" if none) */
const char *tl_last_error(void);
void tl_clear_error(void);
/* library version string */
const char *tl_version(void);
/* sizeof of the public structs, for bindings that mirror them:
 * 0 tl_config_t, 1 tl_solve_info_t, 2 tl_step_record_t, 3 tl_run_options_t,
 * 4 tl_run_result_t, 5 tl_state_t; -1 for an unknown id */
long long tl_sizeof(int which);

/* allocate a chunk for cfg on cfg->cuda_device (all device memory) */
int tl_chunk_create(const tl_config_t *cfg, tl_chunk_t **out);
int tl_chunk_destroy(tl_chunk_t *ch);
/* start.f90:25-112: mesh, states, set_field, then the step-0 field summary */
int tl_start(tl_chunk_t *ch, double *vol, double *mass, double *ie, double *temp);
/* one implicit solve at the chunk's dt (tea_solve.f90:37-509), on the
 * device-resident path; does not advance time */
int tl_timestep(tl_chunk_t *ch, tl_solve_info_t *info);
/* field_summary.f90:27-115 kernel part: sums over the interior */
int tl_field_summary(tl_chunk_t *ch, double *vol, double *mass, double *ie, double *temp);
/* copy a field between the device and a host array in the reference
 * layout; both return once the copy is complete.  A host
 * array in page-locked, mapped memory (cudaHostAlloc, cudaHostRegister) is
 * read or written by the device directly, which on GB300 is several times
 * faster than a copy from pageable memory. */
int tl_get_field(tl_chunk_t *ch, int field, double *host);
int tl_set_field(tl_chunk_t *ch, int field, const double *host);
/* current dt of the chunk (timestep.f90 / calc_dt.f90) */
int tl_set_dt(tl_chunk_t *ch, double dt);
/* number of kernels this chunk has launched so far */
long long tl_kernel_launches(tl_chunk_t *ch);
/* the cudaStream_t all of this chunk's work runs on (for caller-side events) */
void *tl_chunk_stream(tl_chunk_t *ch);
/* per-kernel timing: when on, solves launch kernels one by one (no graph)
 * with a CUDA event pair around each; tl_profile_read returns, per kernel
 * name index idx = 0, 1, ..., the launch count and total milliseconds
 * (TL_ERR_ARG past the last name) */
int tl_set_profiling(tl_chunk_t *ch, int on);
int tl_profile_reset(tl_chunk_t *ch);
/* mixed-precision PPCG: run `steps` (1..5) FP32 inner steps per pass over
 * HBM (temporal blocking; 1 = one kernel per inner step), each CTA taking
 * `seg_strips` 4-row strips of the band-major sequence of (column band,
 * strip) pairs (0: equal shares for one wave of CTAs).  The inner steps
 * give the same bits for every setting.
 * fold_rrn != 0 lets the last fused pass also sum the outer (r - r_store).z,
 * saving a pass over r, r_store and z; that sum then runs in the fused
 * grid's order, so solves with different settings agree to round-off rather
 * than bit for bit (and on GB300 the fold is slower: it adds FP64 work to
 * an issue-bound pass).  Default 5, 0, 0. */
int tl_set_inner_fusion(tl_chunk_t *ch, int steps, int seg_strips, int fold_rrn);
int tl_profile_read(tl_chunk_t *ch, int idx, const char **name, long long *launches, double *ms);
/* the process-wide chunk the reference-named entry points act on */
tl_chunk_t *tl_default_chunk(void);
/* create that chunk from an explicit configuration (initialise_cuda_ does
 * the same from ./tea.in) */
int tl_default_chunk_init(const tl_config_t *cfg);

/* tl_test_fail_alloc -- no counterpart in the reference; a test hook for
 * the allocation-failure paths.  Counting from this call, the nth device
 * allocation the library makes (chunk fields, mixed-precision and warm-start
 * buffers) reports cudaErrorMemoryAllocation without calling cudaMalloc, so
 * the caller sees TL_ERR_ALLOC and everything allocated before it is freed.
 * 0 disarms it.  Returns TL_ERR_ARG for nth < 0. */
int tl_test_fail_alloc(int nth);

/* tl_dot_noalloc -- no counterpart in the reference.  The dot-product
 * reduction of tea_leaf_calc_2norm (sum of a[i]*b[i]) for callers that
 * cannot let the library allocate: hosts that set up their whole
 * device-memory budget once and then run under a fixed cap, hosts whose
 * device memory belongs to another allocator, and hosts that cannot take the
 * device-wide synchronisation of cudaMalloc/cudaFree.  a and b are device
 * pointers to the first element of an nx-by-ny block whose rows are `pitch`
 * elements apart; the sum is written to the device double *result on
 * `stream` (a cudaStream_t, NULL for the default stream), asynchronously.
 * The call allocates nothing: its scratch is a fixed 1 MiB device array
 * held by every GPU that loads the library until the process exits (one
 * partial sum per 32x32 tile, so at most 131040 tiles, about 134 million
 * cells; larger blocks are rejected with TL_ERR_ARG).  The first call on a
 * device looks up that array's address with the device current; make that
 * first call before any stream capture.  All calls share the array: calls
 * that overlap on the GPU race on it and must be ordered by the caller.
 * The looked-up address is kept for the life of the process, so do not reset
 * a device (cudaDeviceReset) while the library is loaded. */
int tl_dot_noalloc(const double *a, const double *b, int nx, int ny, long long pitch,
                   double *result, void *stream);

/* ------------------------------------------------ warm starts
 * No reference counterpart.  With cfg.warm_start set, tl_timestep starts from
 *   u = u^n + sum_i c_i d_i
 * over the last (up to four) increments d_j = u^{n-j+1} - u^{n-j} (none on
 * the first step after tl_start) and, for TL_WARM_LEARNED, a residual
 * network's prediction of the correction A^-1 (u^n - A u^n).  The c_i solve
 * the Galerkin system that minimises the energy 1/2 u.Au - u.u^n, so the
 * start's A-norm error is never above the plain start's; the exit test stays
 * tl_eps * (residual of the plain start u = u^n).
 *
 * The network: six 3x3 convolutions (32 channels, GELU, BF16 tensor-core
 * kernels).  It corrects the increments' own projection u_h: inputs per cell
 * u^n/max|u^n|, log density, log1p Kx, log1p Ky, 100 dt, r_h/max|r_h|,
 * d_1/max|r_h| (r_h = u^n - A u_h); output: (u^{n+1} - u_h)/max|r_h|; the
 * start is then projected jointly over its output and the increments.
 * Parameters: FP32, flat, per layer W[9][coutp][cin]
 * then b[coutp]; layers (cin, coutp) = (16,32) GELU, 4 x (32,32)
 * x + GELU(conv x), (32,16) linear head (output channel 0).  A model file is
 * the 8 bytes "TLWS0001", an int64 parameter count, then the FP32
 * parameters. */
long long tl_warm_start_param_count(void);
/* how the warm start combines its directions: the last `history` (1..8,
 * default 8) increments u^(n-j+1) - u^(n-j), projected in the inner product
 * `projection` (TL_WARM_PROJ_ENERGY, the default, or TL_WARM_PROJ_RESIDUAL).
 * A change restarts the history; a loaded model is kept. */
int tl_set_warm_start_options(tl_chunk_t *ch, int history, int projection);
int tl_set_warm_start_model(tl_chunk_t *ch, const float *params, long long n);
/* training data of the step just solved (which must have run with a warm
 * start, so that the increments are tracked): FP32 [ny][nx][8] at device
 * dst = the seven network inputs and the target (u^{n+1} - u_h)/max|r_h| */
int tl_warm_start_features(tl_chunk_t *ch, float *dst);

/* Network kernels on caller-owned device buffers (NHWC BF16 activations with
 * a one-pixel zero halo, [B][H+2][W+2][C]; W a multiple of 16), used by the
 * trainer.  mode 0: out = GELU(conv(in) + b), pre-activation to pre;
 * 1: out = res + GELU(conv(in) + b); 2: outf[B][H][W] = conv(in)[0] + b[0];
 * 3: out = res + conv(in) (data gradient, weights from tl_nn_pack's wb). */
int tl_nn_conv(int mode, int cin, int coutp, const void *in, const void *w, const float *bias,
               const void *res, void *out, void *pre, float *outf, int B, int H, int W, void *stream);
/* which kernel tl_nn_conv runs: tcgen05 != 0 (the default) the
 * 5th-generation tensor-core kernel (tcgen05.mma, tensor-memory
 * accumulators, 128-pixel tiles), 0 the warp-level mma.sync kernel */
int tl_nn_set_conv_kernel(int tcgen05);
/* TL_OK, or TL_ERR_CUDA (and clears the flag) if a tcgen05 conv since the
 * last call gave up waiting for its tensor-core result (synchronises with
 * the device; the result of that conv is not written) */
int tl_nn_conv_status(void);
int tl_nn_gelu_backward(const void *dh, const void *pre, void *dpre, int C, int B, int H, int W,
                        void *stream);
long long tl_nn_wgrad_partial_floats(int cin, int coutp, int B, int H, int W, int groups_per_cta);
int tl_nn_wgrad(const void *dpre, const void *in, int cin, int coutp, float *partial, float *dw,
                float *db, int B, int H, int W, int groups_per_cta, void *stream);
int tl_nn_adam(float *p, const float *g, float *m, float *v, int n, float lr, float b1, float b2,
               float eps, int step, void *stream);
int tl_nn_pack(const float *w, void *wf, void *wb, int cin, int coutp, void *stream);
int tl_nn_loss(const float *y, const float *t, void *dy, float *partial, int C, int B, int H, int W,
               int margin, void *stream);
int tl_nn_gather(const float *fields, const int *org, void *x, float *t, int F, int C, int Hs, int Ws,
                 int B, int S, void *stream);

/* ------------------------------------------------------- whole program
 * The main program of the reference (tea_leaf.f90 -> start.f90 ->
 * diffuse.f90) restated in C++: read a deck, set up the chunk, run the
 * timestep loop, print the reference's tea.out lines. */
typedef struct tl_step_record {
    int step;
    double time, dt;
    tl_solve_info_t solve;
    int has_summary;
    double vol, mass, ie, temp;
    double wall;                  /* seconds since the first timestep began  */
} tl_step_record_t;

typedef struct tl_run_options {
    const char *out_path;         /* tea.out to write, or NULL               */
    int echo;                     /* also write the log to stdout            */
    int legacy_abi;               /* 1: drive the reference-named entry
                                     points with the host control flow of
                                     tea_solve.f90, as the Fortran does      */
    int max_steps;                /* stop early after this many steps (0: no) */
    tl_step_record_t *records;    /* optional, one per step (step 0 first)   */
    int max_records;
    const char *model_path;       /* warm start model file (tl_warm_start)   */
} tl_run_options_t;

typedef struct tl_run_result {
    int status;
    int steps;
    long long total_iterations;
    double wall_seconds;          /* the whole timestep loop                 */
    double solve_seconds;         /* sum of the implicit solves              */
    double vol, mass, ie, temp;   /* final field summary                     */
    int qa_checked, qa_passed;    /* field_summary.f90:92-112                */
    double qa_diff;
    long long kernel_launches;
    int n_records;
} tl_run_result_t;

int tl_run_deck(const char *deck_text, const tl_run_options_t *opt, tl_run_result_t *res);

/* ------------------------------------------- reference entry points (1) */

/* init_cuda.cu:35 (INITIALISE_ARGS): create the chunk; solver,
 * preconditioner, halo depth, profiler and device come from ./tea.in as in
 * init_cuda.cu:63-163 */
void initialise_cuda_(int *x_min, int *x_max, int *y_min, int *y_max);
/* initialise_chunk_kernel_cuda.cu:28 */
void initialise_chunk_kernel_cuda_(double *d_xmin, double *d_ymin, double *d_dx, double *d_dy);
/* generate_chunk_kernel_cuda.cu:28 */
void generate_chunk_kernel_cuda_(const int *number_of_states, const double *state_density,
                                 const double *state_energy, const double *state_xmin,
                                 const double *state_xmax, const double *state_ymin,
                                 const double *state_ymax, const double *state_radius,
                                 const int *state_geometry, const int *g_rect, const int *g_circ,
                                 const int *g_point);
/* set_field_kernel_cuda.cu:4 */
void set_field_kernel_cuda_(void);
/* field_summary_kernel_cuda.cu:30 */
void field_summary_kernel_cuda_(double *vol, double *mass, double *ie, double *temp);
/* update_halo_kernel_cuda.cu:31 (fields indexed by FIELD_* - 1) */
void update_halo_kernel_cuda_(const int *chunk_neighbours, const int *fields, const int *depth);
/* pack_kernel_cuda.cu:7,14: MPI halo packing; a single chunk has no
 * neighbours, so these only record an error if ever called */
void cuda_pack_buffers_(int *fields, int *offsets, int *depth, int *face, double *host_buffer);
void cuda_unpack_buffers_(int *fields, int *offsets, int *depth, int *face, double *host_buffer);
/* tea_leaf_kernel_cuda.cu:233 (rx, ry are outputs) */
void tea_leaf_common_init_kernel_cuda_(const int *coefficient, double *dt, double *rx,
                                       double *ry, int *zero_boundary, int *reflective_boundary);
/* tea_leaf_kernel_cuda.cu:242 */
void tea_leaf_common_finalise_kernel_cuda_(void);
/* tea_leaf_kernel_cuda.cu:248 */
void tea_leaf_calc_residual_cuda_(void);
/* tea_leaf_kernel_cuda.cu:34 (norm_array 0: u0.u0, 1: r.r, 2: r.z) */
void tea_leaf_calc_2norm_kernel_cuda_(int *norm_array, double *norm);
/* tea_leaf_kernel_cuda.cu:140,146,151,156 */
void tea_leaf_cg_init_kernel_cuda_(double *rro);
void tea_leaf_cg_calc_w_kernel_cuda_(double *pw);
void tea_leaf_cg_calc_ur_kernel_cuda_(double *alpha, double *rrn);
void tea_leaf_cg_calc_p_kernel_cuda_(double *beta);
/* tea_leaf_kernel_cuda.cu:42,50 */
void tea_leaf_cheby_init_kernel_cuda_(const double *ch_alphas, const double *ch_betas,
                                      int *n_coefs, const double *theta);
void tea_leaf_cheby_iterate_kernel_cuda_(const int *cheby_calc_step);
/* tea_leaf_kernel_cuda.cu:301,309,315,322,330,336,342,349,488,503 */
void tea_leaf_ppcg_init_constants_cuda_(const double *ch_alphas, const double *ch_betas,
                                        int *n_inner_steps);
void tea_leaf_ppcg_init_kernel_cuda_(const int *step, double *rro);
void tea_leaf_ppcg_init_sd_kernel_cuda_(const double *theta);
void tea_leaf_ppcg_init_sd_new_kernel_cuda_(const double *theta);
void tea_leaf_ppcg_store_r_kernel_cuda_(void);
void tea_leaf_ppcg_update_z_kernel_cuda_(void);
void tea_leaf_ppcg_calc_rrn_kernel_cuda_(double *norm);
void tea_leaf_ppcg_inner_kernel_cuda_(int *ppcg_cur_step, int *bounds_extra, int *chunk_neighbours);
void tea_leaf_ppcg_calc_2norm_kernel_cuda_(double *norm);
void tea_leaf_ppcg_calc_p_kernel_cuda_(double *beta);
/* tea_leaf_kernel_cuda.cu:215 */
void tea_leaf_jacobi_solve_kernel_cuda_(double *error);

#ifdef __cplusplus
}
#endif
#endif /* TEALEAF_CAPI_H */
