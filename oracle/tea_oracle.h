/*
 * tea_oracle.h -- CPU oracle for the TeaLeaf implicit heat-conduction solve.
 *
 * TEST INFRASTRUCTURE ONLY.  This is a plain-C restatement of the reference
 * algorithm (UK-MAC/TeaLeaf_CUDA: kernel_files/ *.cuknl for the arithmetic,
 * tea_solve.f90 / tea_leaf_cheby.f90 / tea_leaf_ppcg.f90 for control flow,
 * parse.f90 / read_input.f90 for the deck, start.f90 / diffuse.f90 for the
 * main cycle).  It exists to check the CUDA product and to be timed as the
 * CPU baseline; nothing in the product links, imports or calls it.
 *
 * Parity pin: the oracle is checked against the reference's only golden
 * vectors, Benchmarks/tea_bm_{1..4}.out (per-step CG iteration counts and
 * field_summary rows), by tests/test_oracle_golden.py.
 */
#ifndef TEA_ORACLE_H
#define TEA_ORACLE_H

#ifdef __cplusplus
extern "C" {
#endif

#define ORA_MAX_STATES 64

/* solver / preconditioner / coefficient enums: values as data.f90:69-75 and
 * cuda_common.hpp:47-55 */
enum { ORA_JACOBI = 1, ORA_CG = 2, ORA_CHEBY = 3, ORA_PPCG = 4 };
enum { ORA_PREC_NONE = 1, ORA_PREC_DIAG = 2, ORA_PREC_BLOCK = 3 };
enum { ORA_CONDUCTIVITY = 1, ORA_RECIP_CONDUCTIVITY = 2 };
enum { ORA_G_RECT = 1, ORA_G_CIRC = 2, ORA_G_POINT = 3 };

typedef struct {
    int defined;
    double density, energy;
    double xmin, xmax, ymin, ymax, radius;
    int geometry;
} ora_state;

typedef struct {
    int x_cells, y_cells;
    double xmin, xmax, ymin, ymax;
    double dtinit, end_time;
    int end_step, summary_frequency;
    int max_iters;
    double eps;
    int solver, precond, coefficient;
    int halo_depth, reflective, check_result, verbose, profiler_on, test_problem;
    int ch_cg_presteps;
    double ch_cg_epslim;
    int ppcg_inner_steps;
    int nstates;
    ora_state states[ORA_MAX_STATES];
} ora_config;

typedef struct {
    int step;
    double time, dt;
    int iterations;        /* printed "Iteration count" (loop index n - 1) */
    int ppcg_inner_iters;
    double initial_residual;
    double error;          /* |error| at exit */
    double error_ratio;    /* "Conduction error" = error / initial_residual */
    double exact_error_ratio;
    int switch_n;          /* CG iteration at which Chebyshev/PPCG took over */
    int est_itc;
    double eigmin, eigmax;
    int has_summary;
    double vol, mass, ie, temp;
} ora_step_result;

typedef struct ora_chunk ora_chunk;

/* deck text -> config, following parse.f90 + read_input.f90.  Returns 0 on
 * success, a negative code (and a message in err) on a deck error. */
int ora_parse_deck(const char *text, ora_config *cfg, char *err, int errlen);

ora_chunk *ora_chunk_new(const ora_config *cfg);
void ora_chunk_free(ora_chunk *ch);

/* start.f90: initialise_chunk, generate_chunk, set_field, field_summary(0) */
int ora_start(ora_chunk *ch, ora_step_result *summary0);
/* one pass of the diffuse.f90 loop body: timestep + tea_leaf + summary;
 * returns 1 when the run is complete, 0 otherwise */
int ora_step(ora_chunk *ch, ora_step_result *res);

/* field access in the reference layout ((x+2h) x (y+2h), x fastest) */
enum { ORA_F_DENSITY = 1, ORA_F_ENERGY0, ORA_F_ENERGY1, ORA_F_U, ORA_F_P,
       ORA_F_SD, ORA_F_R, ORA_F_U0, ORA_F_W, ORA_F_Z, ORA_F_KX, ORA_F_KY,
       ORA_F_MI, ORA_F_CP, ORA_F_BFP, ORA_F_VOLUME, ORA_F_RTEMP, ORA_F_UTEMP,
       ORA_F_R_STORE };
int ora_get_field(const ora_chunk *ch, int field, double *out);
int ora_set_field(ora_chunk *ch, int field, const double *in);
int ora_field_pitch(const ora_chunk *ch);

/* Per-kernel entry points with the argument meaning of the reference's
 * extern "C" *_kernel_cuda_ symbols (tea_leaf_kernel_cuda.cu), used by the
 * kernel-level parity tests. */
void ora_common_init(ora_chunk *ch, double dt, double *rx, double *ry);
void ora_calc_residual(ora_chunk *ch);
double ora_calc_2norm(ora_chunk *ch, int norm_array);
double ora_cg_init(ora_chunk *ch);
double ora_cg_calc_w(ora_chunk *ch);
double ora_cg_calc_ur(ora_chunk *ch, double alpha);
void ora_cg_calc_p(ora_chunk *ch, double beta);
void ora_cheby_init(ora_chunk *ch, const double *alphas, const double *betas, int n, double theta);
void ora_cheby_iterate(ora_chunk *ch, int step);
void ora_ppcg_init_constants(ora_chunk *ch, const double *alphas, const double *betas, int n);
double ora_ppcg_init(ora_chunk *ch, int step);
void ora_ppcg_init_sd_new(ora_chunk *ch, double theta);
void ora_ppcg_inner(ora_chunk *ch, int step);
void ora_ppcg_store_r(ora_chunk *ch);
void ora_ppcg_update_z(ora_chunk *ch);
double ora_ppcg_calc_rrn(ora_chunk *ch);
double ora_ppcg_calc_zrnorm(ora_chunk *ch);
void ora_ppcg_calc_p(ora_chunk *ch, double beta);
double ora_jacobi_solve(ora_chunk *ch);
void ora_finalise(ora_chunk *ch);
void ora_field_summary(ora_chunk *ch, double *vol, double *mass, double *ie, double *temp);
void ora_update_halo(ora_chunk *ch, const int *fields, int depth);

/* host numerics (tea_leaf_cheby.f90) */
int ora_tqli(double *d, double *e, int n);
int ora_calc_eigenvalues(const double *cg_alphas, const double *cg_betas, int n,
                         double *eigmin, double *eigmax);
void ora_calc_ch_coefs(double *alphas, double *betas, double eigmin, double eigmax,
                       double *theta, int n);

/* number of OpenMP threads the oracle uses (for reporting) */
int ora_num_threads(void);

#ifdef __cplusplus
}
#endif
#endif
