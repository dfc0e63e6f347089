/*
 * tea_oracle.c -- CPU oracle for the TeaLeaf implicit heat-conduction solve.
 *
 * TEST INFRASTRUCTURE ONLY: a plain-C (C11 + OpenMP) restatement of the
 * reference algorithm, used by tests/ as the parity checker and by bench.py as
 * the timed CPU baseline.  The product never links or calls this file.
 *
 * Reference files followed (paths inside UK-MAC/TeaLeaf_CUDA):
 *   deck parsing ............ parse.f90:93-381, read_input.f90:1-329
 *   mesh / states ........... initialise_chunk.f90:27-44,
 *                             kernel_files/initialise_chunk_kernel.cuknl:3-70,
 *                             kernel_files/generate_chunk_kernel.cuknl:5-99,
 *                             generate_chunk_kernel_cuda.cu:50-110
 *   main cycle .............. start.f90:25-112, diffuse.f90:25-101,
 *                             timestep.f90:25-60, calc_dt.f90:25-36
 *   solver control flow ..... tea_solve.f90:37-509
 *   kernels ................. kernel_files/tea_leaf_common.cuknl,
 *                             tea_leaf_cg.cuknl, tea_leaf_cheby.cuknl,
 *                             tea_leaf_ppcg.cuknl, tea_block_jacobi.cuknl,
 *                             tea_leaf_jacobi.cuknl, field_summary_kernel.cuknl
 *   index ranges ............ init_cuda.cu:209-292 (kernel_info_t offsets)
 *   host numerics ........... tea_leaf_cheby.f90:46-220, tea_leaf_ppcg.f90:161-230
 *
 * Arithmetic convention (shared with the CUDA product so that single kernels
 * agree bit for bit): every product-sum that the reference writes as a*b+c is
 * evaluated as one fused multiply-add, the 5-point operator is
 *     diag = (1 + (Ky_n + Ky_c)) + (Kx_e + Kx_c)
 *     Ax   = fma(diag, x_c, -fma(Ky_n, x_n, Ky_c*x_s)) - fma(Kx_e, x_e, Kx_c*x_w)
 * and the file is compiled with -ffp-contract=off so the compiler adds no
 * other contractions.  Dot products are summed per grid row in x order and the
 * row sums in y order, which is deterministic for any thread count.
 *
 * Deviations from the reference CUDA build (each one is a reference defect):
 *   - Chebyshev skips the PPCG re-initialisation block of tea_solve.f90:226-250,
 *     which the reference runs for Chebyshev too and which terminates the CUDA
 *     build (kernel lookup throws, cuda_common.hpp:125-129).
 *   - block-Jacobi strips are truncated at the top boundary when y_cells is not
 *     a multiple of 4 (the reference reads past the tile there).
 *   - the reflective halo update mirrors the interior correctly (the reference
 *     kernel lookup of update_halo_kernel_cuda.cu:51 throws).
 */
#include "tea_oracle.h"

#include <ctype.h>
#include <math.h>
#include <stdint.h>
#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#ifdef _OPENMP
#include <omp.h>
#endif

#define G_SMALL 1.0e-16 /* data.f90:30 */
#define ORA_PAR_MIN 65536 /* grids smaller than this run on one thread */

struct ora_chunk {
    ora_config cfg;
    int nx, ny, h, pitch, rows;
    size_t n2d;
    double *density, *energy0, *energy1, *u, *u0, *p, *r, *w, *z, *mi, *kx, *ky,
        *sd, *rtemp, *utemp, *r_store, *cp, *bfp, *volume, *un;
    double *vertexx, *vertexy, *cellx, *celly, *celldx, *celldy;
    double *rowbuf, *rowbuf2; /* per-row partial sums */
    /* coefficient arrays uploaded by cheby_init / ppcg_init_constants */
    double *ch_alphas_dev, *ch_betas_dev;
    int n_coefs;
    /* driver state (diffuse.f90 / tea_solve.f90 SAVE variables) */
    int step, complete, first;
    double time, dt;
    double eigmin, eigmax, theta, cn;
    double *cg_alphas, *cg_betas, *ch_alphas, *ch_betas;
};

#define IDX(ch, c, r) ((size_t)(c) + (size_t)(r) * (size_t)(ch)->pitch)

int ora_num_threads(void) {
#ifdef _OPENMP
    return omp_get_max_threads();
#else
    return 1;
#endif
}

/* ------------------------------------------------------------------------ */
/* deck parser: parse.f90 (parse_getline :119-237, parse_getword :239-265,  */
/* parse_getival :267-284, parse_getrval :313-335) + read_input.f90         */
/* ------------------------------------------------------------------------ */

typedef struct {
    const char *text;
    size_t pos;
    char line[512];
    char here[512];
    const char *mask;
} deck_reader;

static void set_err(char *err, int errlen, const char *msg, const char *word) {
    if (!err || errlen <= 0) return;
    snprintf(err, (size_t)errlen, "%s%s%s", msg, word ? ": " : "", word ? word : "");
}

/* next raw physical line; returns 0 at end of text */
static int raw_line(deck_reader *d, char *out) {
    if (d->text[d->pos] == '\0') return 0;
    size_t n = 0;
    while (d->text[d->pos] && d->text[d->pos] != '\n') {
        if (n < 100) out[n++] = d->text[d->pos]; /* FMT='(a100)' */
        d->pos++;
    }
    if (d->text[d->pos] == '\n') d->pos++;
    out[n] = '\0';
    return 1;
}

static void rtrim(char *s) {
    size_t n = strlen(s);
    while (n > 0 && s[n - 1] == ' ') s[--n] = '\0';
}

/* parse_getline with dummy=0: returns 0 with d->line filled, -1 at the end of
 * the masked section or of the text */
static int getline_deck(deck_reader *d) {
    char l[512];
    for (;;) {
        if (!raw_line(d, l)) return -1;
        for (char *q = l; *q; ++q) {
            unsigned char c = (unsigned char)*q;
            if (c < 32 || c > 128) *q = ' ';
        }
        char *s = l;
        while (*s == ' ') s++;
        memmove(l, s, strlen(s) + 1);
        char *bang = strchr(l, '!');
        if (bang) *bang = '\0';
        char *semi = strchr(l, ';');
        if (semi) *semi = '\0';
        rtrim(l);
        for (char *q = l; *q; ++q) *q = (char)tolower((unsigned char)*q);
        for (char *q = l; *q; ++q)
            if (*q == '=' || *q == ',') *q = ' ';
        d->line[0] = '\0';
        if (l[0] == '*') {
            char nugget[512];
            size_t k = 0;
            while (l[k] && l[k] != ' ') {
                nugget[k] = l[k];
                k++;
            }
            nugget[k] = '\0';
            if (strncmp(nugget + 1, "end", 3) == 0) {
                char closing[512];
                snprintf(closing, sizeof closing, "*%s", nugget + 4);
                char *last = strrchr(d->here, '*');
                if (last && strcmp(last, closing) == 0) {
                    int was_mask = strcmp(d->here, d->mask) == 0;
                    *last = '\0';
                    if (was_mask) return -1;
                }
            } else {
                strncat(d->here, nugget, sizeof(d->here) - strlen(d->here) - 1);
            }
            continue;
        }
        if (strcmp(d->here, d->mask) == 0 && l[0] != '\0') {
            strcpy(d->line, l);
            return 0;
        }
    }
}

/* parse_getword: next blank-delimited word; with wrap, continue on the next
 * line when this one is exhausted */
static int getword(deck_reader *d, int wrap, char *word) {
    for (;;) {
        char *s = d->line;
        while (*s == ' ') s++;
        size_t k = 0;
        while (s[k] && s[k] != ' ') k++;
        if ((k == 1 && s[0] == '\\') || (k == 0 && wrap)) {
            if (getline_deck(d) != 0) {
                word[0] = '\0';
                return 0;
            }
            continue;
        }
        memcpy(word, s, k);
        word[k] = '\0';
        memmove(d->line, s + k, strlen(s + k) + 1);
        return (int)k;
    }
}

static int getival(const char *word, int *out) {
    char buf[8];
    size_t n = strlen(word);
    if (n > 7) n = 7; /* FMT="(I7)" reads seven characters */
    memcpy(buf, word, n);
    buf[n] = '\0';
    if (n == 0) return -1;
    char *end = NULL;
    long v = strtol(buf, &end, 10);
    if (end == buf || *end != '\0') return -1;
    *out = (int)v;
    return 0;
}

static int getrval(const char *word, double *out) {
    char buf[64];
    size_t n = strlen(word);
    if (n == 0 || n > 40) return -1;
    memcpy(buf, word, n + 1);
    for (char *q = buf; *q; ++q)
        if (*q == 'd') *q = 'e'; /* Fortran double exponent */
    char *end = NULL;
    double v = strtod(buf, &end);
    if (end == buf) return -1;
    if (*end != '\0' && strchr(word, '.') != NULL) return -1;
    *out = v;
    return 0;
}

int ora_parse_deck(const char *text, ora_config *cfg, char *err, int errlen) {
    memset(cfg, 0, sizeof *cfg);
    /* defaults: read_input.f90:38-91 */
    cfg->xmin = 0.0;
    cfg->ymin = 0.0;
    cfg->xmax = 100.0;
    cfg->ymax = 100.0;
    cfg->x_cells = 10;
    cfg->y_cells = 10;
    cfg->end_time = 10.0;
    cfg->end_step = 640000; /* g_ibig */
    cfg->summary_frequency = 10;
    cfg->dtinit = 0.1;
    cfg->max_iters = 1000;
    cfg->eps = 1.0e-10;
    cfg->coefficient = ORA_CONDUCTIVITY;
    cfg->ch_cg_presteps = 25;
    cfg->ch_cg_epslim = 1.0;
    cfg->precond = ORA_PREC_NONE;
    cfg->ppcg_inner_steps = -1;
    cfg->solver = ORA_JACOBI;
    cfg->halo_depth = 1;

    deck_reader d;
    memset(&d, 0, sizeof d);
    d.text = text;
    d.mask = "*tea";
    char word[512];

    /* first pass: number of states (read_input.f90:94-106) */
    int state_max = 0;
    while (getline_deck(&d) == 0) {
        while (getword(&d, 0, word) > 0) {
            if (strcmp(word, "state") == 0) {
                int s;
                getword(&d, 1, word);
                if (getival(word, &s) != 0) {
                    set_err(err, errlen, "Error attempting to convert to integer", word);
                    return -2;
                }
                if (s > state_max) state_max = s;
                break;
            }
        }
    }
    if (state_max < 1) {
        set_err(err, errlen, "No states defined.", NULL);
        return -1;
    }
    if (state_max > ORA_MAX_STATES) {
        set_err(err, errlen, "Too many states", NULL);
        return -1;
    }
    cfg->nstates = state_max;

    memset(&d, 0, sizeof d);
    d.text = text;
    d.mask = "*tea";
#define RVAL(dst)                                                                  \
    do {                                                                           \
        getword(&d, 1, word);                                                      \
        if (getrval(word, &(dst)) != 0) {                                          \
            set_err(err, errlen, "Error attempting to convert to real", word);    \
            return -2;                                                             \
        }                                                                          \
    } while (0)
#define IVAL(dst)                                                                  \
    do {                                                                           \
        getword(&d, 1, word);                                                      \
        if (getival(word, &(dst)) != 0) {                                          \
            set_err(err, errlen, "Error attempting to convert to integer", word); \
            return -2;                                                             \
        }                                                                          \
    } while (0)

    while (getline_deck(&d) == 0) {
        while (getword(&d, 0, word) > 0) {
            if (!strcmp(word, "initial_timestep")) RVAL(cfg->dtinit);
            else if (!strcmp(word, "end_time")) RVAL(cfg->end_time);
            else if (!strcmp(word, "end_step")) IVAL(cfg->end_step);
            else if (!strcmp(word, "xmin")) RVAL(cfg->xmin);
            else if (!strcmp(word, "xmax")) RVAL(cfg->xmax);
            else if (!strcmp(word, "ymin")) RVAL(cfg->ymin);
            else if (!strcmp(word, "ymax")) RVAL(cfg->ymax);
            else if (!strcmp(word, "x_cells")) IVAL(cfg->x_cells);
            else if (!strcmp(word, "y_cells")) IVAL(cfg->y_cells);
            else if (!strcmp(word, "visit_frequency")) { int v; IVAL(v); (void)v; }
            else if (!strcmp(word, "summary_frequency")) IVAL(cfg->summary_frequency);
            else if (!strcmp(word, "tl_ch_cg_presteps")) IVAL(cfg->ch_cg_presteps);
            else if (!strcmp(word, "tl_ppcg_inner_steps")) IVAL(cfg->ppcg_inner_steps);
            else if (!strcmp(word, "tl_ch_cg_epslim")) RVAL(cfg->ch_cg_epslim);
            else if (!strcmp(word, "tl_check_result")) cfg->check_result = 1;
            else if (!strcmp(word, "tl_preconditioner_type")) {
                while (getword(&d, 0, word) > 0) {
                    if (!strcmp(word, "none")) cfg->precond = ORA_PREC_NONE;
                    else if (!strcmp(word, "jac_diag")) cfg->precond = ORA_PREC_DIAG;
                    else if (!strcmp(word, "jac_block")) cfg->precond = ORA_PREC_BLOCK;
                    else {
                        set_err(err, errlen, "Invalid preconditioner type specified", word);
                        return -3;
                    }
                }
            }
            else if (!strcmp(word, "use_cuda_kernels")) { }
            else if (!strcmp(word, "verbose_on")) cfg->verbose = 1;
            else if (!strcmp(word, "tl_use_jacobi")) cfg->solver = ORA_JACOBI;
            else if (!strcmp(word, "tl_use_cg")) cfg->solver = ORA_CG;
            else if (!strcmp(word, "tl_use_ppcg")) cfg->solver = ORA_PPCG;
            else if (!strcmp(word, "tl_use_chebyshev")) cfg->solver = ORA_CHEBY;
            else if (!strcmp(word, "reflective_boundary")) cfg->reflective = 1;
            else if (!strcmp(word, "profiler_on")) cfg->profiler_on = 1;
            else if (!strcmp(word, "halo_depth")) {
                IVAL(cfg->halo_depth);
                if (cfg->halo_depth < 1) {
                    set_err(err, errlen, "Invalid halo exchange depth specified", NULL);
                    return -4;
                }
            }
            else if (!strcmp(word, "tl_max_iters")) IVAL(cfg->max_iters);
            else if (!strcmp(word, "tl_eps")) RVAL(cfg->eps);
            else if (!strcmp(word, "tl_coefficient_density")) cfg->coefficient = ORA_CONDUCTIVITY;
            else if (!strcmp(word, "tl_coefficient_inverse_density")) cfg->coefficient = ORA_RECIP_CONDUCTIVITY;
            else if (!strcmp(word, "test_problem")) IVAL(cfg->test_problem);
            else if (!strcmp(word, "state")) {
                int s;
                IVAL(s);
                if (s < 1 || s > cfg->nstates) {
                    set_err(err, errlen, "Invalid state number", word);
                    return -5;
                }
                ora_state *st = &cfg->states[s - 1];
                if (st->defined) {
                    set_err(err, errlen, "State defined twice.", NULL);
                    return -5;
                }
                st->defined = 1;
                while (getword(&d, 0, word) > 0) {
                    if (!strcmp(word, "xmin")) RVAL(st->xmin);
                    else if (!strcmp(word, "ymin")) RVAL(st->ymin);
                    else if (!strcmp(word, "xmax")) RVAL(st->xmax);
                    else if (!strcmp(word, "ymax")) RVAL(st->ymax);
                    else if (!strcmp(word, "radius")) RVAL(st->radius);
                    else if (!strcmp(word, "density")) RVAL(st->density);
                    else if (!strcmp(word, "energy")) RVAL(st->energy);
                    else if (!strcmp(word, "geometry")) {
                        getword(&d, 1, word);
                        if (!strcmp(word, "rectangle")) st->geometry = ORA_G_RECT;
                        else if (!strcmp(word, "circle")) st->geometry = ORA_G_CIRC;
                        else if (!strcmp(word, "point")) st->geometry = ORA_G_POINT;
                    }
                }
            }
        }
    }
#undef RVAL
#undef IVAL

    /* read_input.f90:294-297: default inner steps from the grid, in REAL(4) */
    if (cfg->ppcg_inner_steps == -1) {
        float cells = (float)(cfg->x_cells * cfg->y_cells);
        cfg->ppcg_inner_steps = 4 * (int)sqrtf(sqrtf(cells));
    }
    /* read_input.f90:299-301 */
    if (cfg->halo_depth > 1 && cfg->precond == ORA_PREC_BLOCK && cfg->solver == ORA_PPCG) {
        set_err(err, errlen, "Unable to use nonstandard halo depth with block jacobi preconditioner", NULL);
        return -6;
    }
    /* read_input.f90:320-327: states 2..N shrunk by a hundredth of a cell */
    double dx = (cfg->xmax - cfg->xmin) / (double)(float)cfg->x_cells;
    double dy = (cfg->ymax - cfg->ymin) / (double)(float)cfg->y_cells;
    for (int n = 1; n < cfg->nstates; ++n) {
        cfg->states[n].xmin += dx / 100.0;
        cfg->states[n].ymin += dy / 100.0;
        cfg->states[n].xmax -= dx / 100.0;
        cfg->states[n].ymax -= dy / 100.0;
    }
    return 0;
}

/* ------------------------------------------------------------------------ */
/* chunk                                                                    */
/* ------------------------------------------------------------------------ */

static double *zalloc(size_t n) {
    double *p = (double *)calloc(n ? n : 1, sizeof(double));
    return p;
}

ora_chunk *ora_chunk_new(const ora_config *cfg) {
    ora_chunk *ch = (ora_chunk *)calloc(1, sizeof *ch);
    if (!ch) return NULL;
    ch->cfg = *cfg;
    ch->nx = cfg->x_cells;
    ch->ny = cfg->y_cells;
    ch->h = cfg->halo_depth;
    ch->pitch = ch->nx + 2 * ch->h;
    ch->rows = ch->ny + 2 * ch->h;
    ch->n2d = (size_t)ch->pitch * (size_t)ch->rows;
    double **arrays[] = {&ch->density, &ch->energy0, &ch->energy1, &ch->u, &ch->u0, &ch->p,
                         &ch->r, &ch->w, &ch->z, &ch->mi, &ch->kx, &ch->ky, &ch->sd,
                         &ch->rtemp, &ch->utemp, &ch->r_store, &ch->cp, &ch->bfp,
                         &ch->volume, &ch->un};
    for (size_t i = 0; i < sizeof arrays / sizeof arrays[0]; ++i) {
        *arrays[i] = zalloc(ch->n2d);
        if (!*arrays[i]) { ora_chunk_free(ch); return NULL; }
    }
    ch->vertexx = zalloc((size_t)ch->pitch + 1);
    ch->vertexy = zalloc((size_t)ch->rows + 1);
    ch->cellx = zalloc((size_t)ch->pitch);
    ch->celly = zalloc((size_t)ch->rows);
    ch->celldx = zalloc((size_t)ch->pitch);
    ch->celldy = zalloc((size_t)ch->rows);
    ch->rowbuf = zalloc((size_t)ch->rows);
    ch->rowbuf2 = zalloc((size_t)ch->rows);
    size_t mi = (size_t)cfg->max_iters + 4;
    ch->cg_alphas = zalloc(mi);
    ch->cg_betas = zalloc(mi);
    size_t nc = mi > (size_t)cfg->ppcg_inner_steps + 4 ? mi : (size_t)cfg->ppcg_inner_steps + 4;
    ch->ch_alphas = zalloc(nc);
    ch->ch_betas = zalloc(nc);
    ch->ch_alphas_dev = zalloc(nc);
    ch->ch_betas_dev = zalloc(nc);
    ch->first = 1;
    return ch;
}

void ora_chunk_free(ora_chunk *ch) {
    if (!ch) return;
    double *all[] = {ch->density, ch->energy0, ch->energy1, ch->u, ch->u0, ch->p, ch->r,
                     ch->w, ch->z, ch->mi, ch->kx, ch->ky, ch->sd, ch->rtemp, ch->utemp,
                     ch->r_store, ch->cp, ch->bfp, ch->volume, ch->un, ch->vertexx,
                     ch->vertexy, ch->cellx, ch->celly, ch->celldx, ch->celldy,
                     ch->rowbuf, ch->rowbuf2, ch->cg_alphas, ch->cg_betas,
                     ch->ch_alphas, ch->ch_betas, ch->ch_alphas_dev, ch->ch_betas_dev};
    for (size_t i = 0; i < sizeof all / sizeof all[0]; ++i) free(all[i]);
    free(ch);
}

int ora_field_pitch(const ora_chunk *ch) { return ch->pitch; }

static double *field_ptr(const ora_chunk *ch, int f) {
    switch (f) {
    case ORA_F_DENSITY: return ch->density;
    case ORA_F_ENERGY0: return ch->energy0;
    case ORA_F_ENERGY1: return ch->energy1;
    case ORA_F_U: return ch->u;
    case ORA_F_P: return ch->p;
    case ORA_F_SD: return ch->sd;
    case ORA_F_R: return ch->r;
    case ORA_F_U0: return ch->u0;
    case ORA_F_W: return ch->w;
    case ORA_F_Z: return ch->z;
    case ORA_F_KX: return ch->kx;
    case ORA_F_KY: return ch->ky;
    case ORA_F_MI: return ch->mi;
    case ORA_F_CP: return ch->cp;
    case ORA_F_BFP: return ch->bfp;
    case ORA_F_VOLUME: return ch->volume;
    case ORA_F_RTEMP: return ch->rtemp;
    case ORA_F_UTEMP: return ch->utemp;
    case ORA_F_R_STORE: return ch->r_store;
    default: return NULL;
    }
}

int ora_get_field(const ora_chunk *ch, int field, double *out) {
    double *f = field_ptr(ch, field);
    if (!f) return -1;
    memcpy(out, f, ch->n2d * sizeof(double));
    return 0;
}

int ora_set_field(ora_chunk *ch, int field, const double *in) {
    double *f = field_ptr(ch, field);
    if (!f) return -1;
    memcpy(f, in, ch->n2d * sizeof(double));
    return 0;
}

/* ------------------------------------------------------------------------ */
/* deterministic sums: per row in x order, then rows in y order              */
/* ------------------------------------------------------------------------ */

static double sum_rows(const ora_chunk *ch, const double *rowbuf) {
    double s = 0.0;
    for (int k = ch->h; k < ch->h + ch->ny; ++k) s += rowbuf[k];
    return s;
}

/* the 5-point operator of tea_leaf_common.cuknl:28-34 */
static inline double smvp(const ora_chunk *ch, const double *x, size_t i) {
    const double *kx = ch->kx, *ky = ch->ky;
    const size_t P = (size_t)ch->pitch;
    double diag = (1.0 + (ky[i + P] + ky[i])) + (kx[i + 1] + kx[i]);
    double a = fma(ky[i + P], x[i + P], ky[i] * x[i - P]);
    double b = fma(kx[i + 1], x[i + 1], kx[i] * x[i - 1]);
    return fma(diag, x[i], -a) - b;
}

static inline double diag_of(const ora_chunk *ch, size_t i) {
    const size_t P = (size_t)ch->pitch;
    return (1.0 + (ch->ky[i + P] + ch->ky[i])) + (ch->kx[i + 1] + ch->kx[i]);
}

/* ------------------------------------------------------------------------ */
/* mesh, states, main-cycle kernels                                         */
/* ------------------------------------------------------------------------ */

/* initialise_chunk.f90:33-43 + initialise_chunk_kernel.cuknl:3-70 */
static void initialise_chunk(ora_chunk *ch) {
    const ora_config *c = &ch->cfg;
    double dx = (c->xmax - c->xmin) / (double)(float)c->x_cells;
    double dy = (c->ymax - c->ymin) / (double)(float)c->y_cells;
    double xmin = c->xmin, ymin = c->ymin;
    int h = ch->h;
    for (int col = 0; col <= ch->nx + 2 * h; ++col) {
        ch->vertexx[col] = xmin + dx * (double)(col - h);
        if (col < ch->pitch) {
            double plus = xmin + dx * (double)(col - h + 1);
            ch->cellx[col] = 0.5 * (ch->vertexx[col] + plus);
            ch->celldx[col] = dx;
        }
    }
    for (int row = 0; row <= ch->ny + 2 * h; ++row) {
        ch->vertexy[row] = ymin + dy * (double)(row - h);
        if (row < ch->rows) {
            double plus = ymin + dy * (double)(row - h + 1);
            ch->celly[row] = 0.5 * (ch->vertexy[row] + plus);
            ch->celldy[row] = dy;
        }
    }
    for (size_t i = 0; i < ch->n2d; ++i) ch->volume[i] = dx * dy;
}

/* generate_chunk_kernel.cuknl:5-99, launched per state as in
 * generate_chunk_kernel_cuda.cu:86-98 over the interior range */
static void generate_chunk(ora_chunk *ch) {
    const ora_config *c = &ch->cfg;
    int h = ch->h;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->energy0[i] = c->states[0].energy;
            ch->density[i] = c->states[0].density;
        }
    for (int s = 1; s < c->nstates; ++s) {
        const ora_state *st = &c->states[s];
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
        for (int row = h; row < h + ch->ny; ++row)
            for (int col = h; col < h + ch->nx; ++col) {
                size_t i = IDX(ch, col, row);
                int hit = 0;
                if (st->geometry == ORA_G_RECT) {
                    hit = ch->vertexx[col + 1] >= st->xmin && ch->vertexx[col] < st->xmax &&
                          ch->vertexy[row + 1] >= st->ymin && ch->vertexy[row] < st->ymax;
                } else if (st->geometry == ORA_G_CIRC) {
                    double xp = ch->cellx[col] - st->xmin;
                    double yp = ch->celly[row] - st->ymin;
                    double rad = sqrt(xp * xp + yp * yp);
                    hit = rad <= st->radius;
                } else if (st->geometry == ORA_G_POINT) {
                    hit = ch->vertexx[col] == st->xmin && ch->vertexy[row] == st->ymin;
                }
                if (hit) {
                    ch->energy0[i] = st->energy;
                    ch->density[i] = st->density;
                }
            }
    }
    /* generate_chunk_init_u(energy0): u = u0 = energy*density */
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->u[i] = ch->energy0[i] * ch->density[i];
            ch->u0[i] = ch->energy0[i] * ch->density[i];
        }
}

/* reflective external boundary, TeaLeaf's mirror semantics (the intent of
 * update_halo_kernel.cuknl:5-96): halo row h-1-k <- interior row h+k, etc. */
static void reflect_field(ora_chunk *ch, double *f, int depth) {
    int h = ch->h, nx = ch->nx, ny = ch->ny;
    if (depth > h) depth = h;
    for (int k = 0; k < depth; ++k)
        for (int col = h - depth; col < h + nx + depth; ++col) {
            f[IDX(ch, col, h - 1 - k)] = f[IDX(ch, col, h + k)];
            f[IDX(ch, col, h + ny + k)] = f[IDX(ch, col, h + ny - 1 - k)];
        }
    for (int k = 0; k < depth; ++k)
        for (int row = h - depth; row < h + ny + depth; ++row) {
            f[IDX(ch, h - 1 - k, row)] = f[IDX(ch, h + k, row)];
            f[IDX(ch, h + nx + k, row)] = f[IDX(ch, h + nx - 1 - k, row)];
        }
}

/* update_halo.f90:30-68: the single-chunk exchange is a no-op; the external
 * boundary update runs only with reflective_boundary.  fields[] is indexed by
 * FIELD_* - 1 (data.f90:44-50). */
void ora_update_halo(ora_chunk *ch, const int *fields, int depth) {
    if (!ch->cfg.reflective) return;
    double *f[7] = {ch->density, ch->energy0, ch->energy1, ch->u, ch->p, ch->sd, ch->r};
    for (int k = 0; k < 7; ++k)
        if (fields[k]) reflect_field(ch, f[k], depth);
}

static void halo1(ora_chunk *ch, int field, int depth) {
    int fl[7] = {0};
    fl[field - 1] = 1;
    ora_update_halo(ch, fl, depth);
}

/* set_field_kernel.cuknl:5-16 */
static void set_field(ora_chunk *ch) {
    int h = ch->h;
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->energy1[i] = ch->energy0[i];
        }
}

/* field_summary_kernel.cuknl:5-58 (energy1, field_summary_kernel_cuda.cu:39) */
void ora_field_summary(ora_chunk *ch, double *vol, double *mass, double *ie, double *temp) {
    int h = ch->h;
    double *rb[4];
    for (int k = 0; k < 4; ++k) rb[k] = zalloc((size_t)ch->rows);
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row) {
        double v = 0, m = 0, e = 0, t = 0;
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            double cv = ch->volume[i];
            double cm = cv * ch->density[i];
            v += cv;
            m += cm;
            e += cm * ch->energy1[i];
            t += cm * ch->u[i];
        }
        rb[0][row] = v;
        rb[1][row] = m;
        rb[2][row] = e;
        rb[3][row] = t;
    }
    *vol = sum_rows(ch, rb[0]);
    *mass = sum_rows(ch, rb[1]);
    *ie = sum_rows(ch, rb[2]);
    *temp = sum_rows(ch, rb[3]);
    for (int k = 0; k < 4; ++k) free(rb[k]);
}

/* ------------------------------------------------------------------------ */
/* solver kernels                                                           */
/* ------------------------------------------------------------------------ */

/* tea_leaf_kernel_cuda.cu:254-283: calcrxry, init_common, zero_boundaries,
 * generate_chunk_init_u(energy1) */
void ora_common_init(ora_chunk *ch, double dt, double *rx_out, double *ry_out) {
    int h = ch->h, nx = ch->nx, ny = ch->ny;
    double dx = ch->celldx[h], dy = ch->celldy[h];
    double rx = dt / (dx * dx), ry = dt / (dy * dy);
    if (rx_out) *rx_out = rx;
    if (ry_out) *ry_out = ry;
    const int recip = ch->cfg.coefficient == ORA_RECIP_CONDUCTIVITY;
    const size_t P = (size_t)ch->pitch;
    /* device_tea_leaf_init_common over columns h..nx+2h-1, rows h..ny+2h-1
     * (tea_leaf_common.cuknl:60-97, range init_cuda.cu:290) */
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < ny + 2 * h; ++row)
        for (int col = h; col < nx + 2 * h; ++col) {
            size_t i = IDX(ch, col, row);
            double dc, dl, dd;
            if (!recip) {
                dc = ch->density[i];
                dl = ch->density[i - 1];
                dd = ch->density[i - P];
            } else {
                dc = 1.0 / ch->density[i];
                dl = 1.0 / ch->density[i - 1];
                dd = 1.0 / ch->density[i - P];
            }
            double kx = (dl + dc) / (2.0 * dl * dc);
            double ky = (dd + dc) / (2.0 * dd * dc);
            ch->kx[i] = kx * rx;
            ch->ky[i] = ky * ry;
        }
    /* device_tea_leaf_zero_boundaries (tea_leaf_common.cuknl:99-129): all four
     * faces are external on one chunk, so every boundary face is zeroed
     * unless the boundary is reflective */
    if (!ch->cfg.reflective) {
        for (int row = 0; row < ch->rows; ++row)
            for (int col = 0; col < ch->pitch; ++col) {
                size_t i = IDX(ch, col, row);
                if (col <= h || col > nx - 1 + h) ch->kx[i] = 0.0;
                if (row <= h || row > ny - 1 + h) ch->ky[i] = 0.0;
            }
    }
    /* generate_chunk_init_u(energy1) */
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ny; ++row)
        for (int col = h; col < h + nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->u[i] = ch->energy1[i] * ch->density[i];
            ch->u0[i] = ch->energy1[i] * ch->density[i];
        }
}

/* tea_leaf_common.cuknl:19-39 */
void ora_calc_residual(ora_chunk *ch) {
    int h = ch->h;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->r[i] = ch->u0[i] - smvp(ch, ch->u, i);
        }
}

static double dot(ora_chunk *ch, const double *a, const double *b) {
    int h = ch->h;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row) {
        double s = 0.0;
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            s = fma(a[i], b[i], s);
        }
        ch->rowbuf[row] = s;
    }
    return sum_rows(ch, ch->rowbuf);
}

/* tea_leaf_kernel_cuda.cu:56-87 */
double ora_calc_2norm(ora_chunk *ch, int norm_array) {
    if (norm_array == 0) return dot(ch, ch->u0, ch->u0);
    if (norm_array == 1) return dot(ch, ch->r, ch->r);
    if (ch->cfg.precond != ORA_PREC_NONE) return dot(ch, ch->r, ch->z);
    return dot(ch, ch->r, ch->r);
}

/* block-Jacobi strips: tea_block_jacobi.cuknl:5-7 coefficients,
 * block_init :83-111, block_solve_func :11-46.  Strips are 4 rows high and
 * start at interior rows 0, 4, 8, ...; the last strip is truncated at the top
 * boundary. */
#define STRIP 4
static void block_init(ora_chunk *ch) {
    int h = ch->h, ny = ch->ny;
    const size_t P = (size_t)ch->pitch;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int s0 = 0; s0 < ny; s0 += STRIP) {
        int m = ny - s0 < STRIP ? ny - s0 : STRIP;
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i0 = IDX(ch, col, h + s0);
            /* cp[0] = c0/b0 with c = -Ky(k+1), b = diag */
            ch->cp[i0] = (-ch->ky[i0 + P]) / diag_of(ch, i0);
            for (int k = 1; k < m; ++k) {
                size_t i = i0 + (size_t)k * P;
                /* bfp = 1/(b - a*cp[k-1]) with a = -Ky(k) */
                ch->bfp[i] = 1.0 / fma(ch->ky[i], ch->cp[i - P], diag_of(ch, i));
                ch->cp[i] = (-ch->ky[i + P]) * ch->bfp[i];
            }
        }
    }
}

/* z = M^-1 x on the strip containing interior row s0.. (x in registers) */
static inline void strip_solve(const ora_chunk *ch, size_t i0, int m, const double *x, double *zout) {
    const size_t P = (size_t)ch->pitch;
    double dp[STRIP];
    dp[0] = x[0] / diag_of(ch, i0);
    for (int k = 1; k < m; ++k) {
        size_t i = i0 + (size_t)k * P;
        dp[k] = fma(ch->ky[i], dp[k - 1], x[k]) * ch->bfp[i];
    }
    zout[m - 1] = dp[m - 1];
    for (int k = m - 2; k >= 0; --k) {
        size_t i = i0 + (size_t)k * P;
        zout[k] = fma(-ch->cp[i], zout[k + 1], dp[k]);
    }
}

/* z = M^-1 src over the whole grid for the block preconditioner */
static void block_solve(ora_chunk *ch, const double *src, double *dst) {
    int h = ch->h, ny = ch->ny;
    const size_t P = (size_t)ch->pitch;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int s0 = 0; s0 < ny; s0 += STRIP) {
        int m = ny - s0 < STRIP ? ny - s0 : STRIP;
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i0 = IDX(ch, col, h + s0);
            double x[STRIP], zz[STRIP];
            for (int k = 0; k < m; ++k) x[k] = src[i0 + (size_t)k * P];
            strip_solve(ch, i0, m, x, zz);
            for (int k = 0; k < m; ++k) dst[i0 + (size_t)k * P] = zz[k];
        }
    }
}

/* tea_leaf_common.cuknl:131-147 */
static void init_jac_diag(ora_chunk *ch) {
    int h = ch->h;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->mi[i] = 1.0 / diag_of(ch, i);
        }
}

/* tea_leaf_kernel_cuda.cu:164-186 + tea_leaf_cg.cuknl:5-39 */
double ora_cg_init(ora_chunk *ch) {
    int h = ch->h, pc = ch->cfg.precond;
    if (pc == ORA_PREC_BLOCK) {
        block_init(ch);
        block_solve(ch, ch->r, ch->z);
    } else if (pc == ORA_PREC_DIAG) {
        init_jac_diag(ch);
    }
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row) {
        double s = 0.0;
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            if (pc == ORA_PREC_BLOCK) {
                ch->p[i] = ch->z[i];
            } else if (pc == ORA_PREC_DIAG) {
                ch->z[i] = ch->r[i] * ch->mi[i];
                ch->p[i] = ch->z[i];
            } else {
                ch->p[i] = ch->r[i];
            }
            s = fma(ch->r[i], ch->p[i], s);
        }
        ch->rowbuf[row] = s;
    }
    return sum_rows(ch, ch->rowbuf);
}

/* tea_leaf_cg.cuknl:43-68 */
double ora_cg_calc_w(ora_chunk *ch) {
    int h = ch->h;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row) {
        double s = 0.0;
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->w[i] = smvp(ch, ch->p, i);
            s = fma(ch->p[i], ch->w[i], s);
        }
        ch->rowbuf[row] = s;
    }
    return sum_rows(ch, ch->rowbuf);
}

/* tea_leaf_cg.cuknl:72-137 */
double ora_cg_calc_ur(ora_chunk *ch, double alpha) {
    int h = ch->h, pc = ch->cfg.precond;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->u[i] = fma(alpha, ch->p[i], ch->u[i]);
            ch->r[i] = fma(-alpha, ch->w[i], ch->r[i]);
        }
    if (pc == ORA_PREC_BLOCK) {
        block_solve(ch, ch->r, ch->z);
        return dot(ch, ch->r, ch->z);
    }
    if (pc == ORA_PREC_DIAG) {
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
        for (int row = h; row < h + ch->ny; ++row) {
            double s = 0.0;
            for (int col = h; col < h + ch->nx; ++col) {
                size_t i = IDX(ch, col, row);
                ch->z[i] = ch->r[i] * ch->mi[i];
                s = fma(ch->r[i], ch->z[i], s);
            }
            ch->rowbuf[row] = s;
        }
        return sum_rows(ch, ch->rowbuf);
    }
    return dot(ch, ch->r, ch->r);
}

/* tea_leaf_cg.cuknl:141-161 */
void ora_cg_calc_p(ora_chunk *ch, double beta) {
    int h = ch->h;
    const double *src = ch->cfg.precond != ORA_PREC_NONE ? ch->z : ch->r;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->p[i] = fma(beta, ch->p[i], src[i]);
        }
}

/* the device copy of the Chebyshev / PPCG coefficients
 * (tea_leaf_kernel_cuda.cu:89-104) */
static void upload_coefs(ora_chunk *ch, const double *a, const double *b, int n) {
    memcpy(ch->ch_alphas_dev, a, (size_t)n * sizeof(double));
    memcpy(ch->ch_betas_dev, b, (size_t)n * sizeof(double));
    ch->n_coefs = n;
}

/* tea_leaf_cheby.cuknl:5-68 (init_p) and :71-82 (calc_u) */
void ora_cheby_init(ora_chunk *ch, const double *alphas, const double *betas, int n, double theta) {
    int h = ch->h, pc = ch->cfg.precond;
    upload_coefs(ch, alphas, betas, n);
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->w[i] = smvp(ch, ch->u, i);
            ch->r[i] = ch->u0[i] - ch->w[i];
        }
    if (pc == ORA_PREC_BLOCK) block_solve(ch, ch->r, ch->un);
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            if (pc == ORA_PREC_BLOCK) ch->p[i] = ch->un[i] / theta;
            else if (pc == ORA_PREC_DIAG) ch->p[i] = (ch->mi[i] * ch->r[i]) / theta;
            else ch->p[i] = ch->r[i] / theta;
            ch->u[i] += ch->p[i];
        }
}

/* tea_leaf_kernel_cuda.cu:124-135 + tea_leaf_cheby.cuknl:84-152, :71-82.
 * step is the 1-based Chebyshev step; coefficient index step-1 */
void ora_cheby_iterate(ora_chunk *ch, int step) {
    int h = ch->h, pc = ch->cfg.precond;
    double al = ch->ch_alphas_dev[step - 1], be = ch->ch_betas_dev[step - 1];
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->w[i] = smvp(ch, ch->u, i);
            ch->r[i] = ch->u0[i] - ch->w[i];
        }
    if (pc == ORA_PREC_BLOCK) block_solve(ch, ch->r, ch->un);
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            if (pc == ORA_PREC_BLOCK) ch->p[i] = fma(al, ch->p[i], be * ch->un[i]);
            else if (pc == ORA_PREC_DIAG) ch->p[i] = fma(al, ch->p[i], (be * ch->mi[i]) * ch->r[i]);
            else ch->p[i] = fma(al, ch->p[i], be * ch->r[i]);
            ch->u[i] += ch->p[i];
        }
}

void ora_ppcg_init_constants(ora_chunk *ch, const double *alphas, const double *betas, int n) {
    upload_coefs(ch, alphas, betas, n);
}

/* tea_leaf_ppcg.cuknl:319-420.  step 1: p = z = 0 then z = M^-1 r, p = z (or
 * p = r without a preconditioner); step 2: z = M^-1 r only; step 3: p = z.
 * Steps 1 and 3 return sum r.p, step 2 returns 0. */
double ora_ppcg_init(ora_chunk *ch, int step) {
    int h = ch->h, pc = ch->cfg.precond;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            if (step == 1) {
                ch->p[i] = 0.0;
                ch->z[i] = 0.0;
            } else if (step == 3) {
                ch->p[i] = 0.0;
            }
        }
    if (pc != ORA_PREC_NONE || step == 3) {
        if (step == 1 || step == 2) {
            if (pc == ORA_PREC_BLOCK) {
                block_solve(ch, ch->r, ch->z);
            } else if (pc == ORA_PREC_DIAG) {
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
                for (int row = h; row < h + ch->ny; ++row)
                    for (int col = h; col < h + ch->nx; ++col) {
                        size_t i = IDX(ch, col, row);
                        ch->z[i] = ch->mi[i] * ch->r[i];
                    }
            }
        }
        if (step == 1 || step == 3) {
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
            for (int row = h; row < h + ch->ny; ++row)
                for (int col = h; col < h + ch->nx; ++col) {
                    size_t i = IDX(ch, col, row);
                    ch->p[i] = ch->z[i];
                }
        }
    } else if (step == 1) {
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
        for (int row = h; row < h + ch->ny; ++row)
            for (int col = h; col < h + ch->nx; ++col) {
                size_t i = IDX(ch, col, row);
                ch->p[i] = ch->r[i];
            }
    }
    if (step == 1 || step == 3) return dot(ch, ch->r, ch->p);
    return 0.0;
}

/* tea_leaf_ppcg.cuknl:58-89 */
void ora_ppcg_init_sd_new(ora_chunk *ch, double theta) {
    int h = ch->h, pc = ch->cfg.precond;
    double theta_r = 1.0 / theta;
    const double *src = pc != ORA_PREC_NONE ? ch->z : ch->r;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->sd[i] = src[i] * theta_r;
            ch->rtemp[i] = ch->r[i];
            ch->utemp[i] = ch->sd[i];
        }
}

/* one inner step: tea_leaf_ppcg.cuknl:154-173 (update_r) then :178-244
 * (calc_sd_new) with coefficient index step-1 (tea_leaf_kernel_cuda.cu:418-486) */
void ora_ppcg_inner(ora_chunk *ch, int step) {
    int h = ch->h, pc = ch->cfg.precond;
    double al = ch->ch_alphas_dev[step - 1], be = ch->ch_betas_dev[step - 1];
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->rtemp[i] -= smvp(ch, ch->sd, i);
        }
    if (pc == ORA_PREC_BLOCK) block_solve(ch, ch->rtemp, ch->un);
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            if (pc == ORA_PREC_BLOCK) ch->sd[i] = fma(al, ch->sd[i], be * ch->un[i]);
            else if (pc == ORA_PREC_DIAG) ch->sd[i] = fma(al, ch->sd[i], (be * ch->rtemp[i]) * ch->mi[i]);
            else ch->sd[i] = fma(al, ch->sd[i], be * ch->rtemp[i]);
            ch->utemp[i] += ch->sd[i];
        }
}

void ora_ppcg_store_r(ora_chunk *ch) {
    int h = ch->h;
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->r_store[i] = ch->r[i];
        }
}

void ora_ppcg_update_z(ora_chunk *ch) {
    int h = ch->h;
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->z[i] = ch->utemp[i];
        }
}

/* tea_leaf_ppcg.cuknl:279-297: sum (r - r_store) * z */
double ora_ppcg_calc_rrn(ora_chunk *ch) {
    int h = ch->h;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row) {
        double s = 0.0;
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            s = fma(ch->r[i] - ch->r_store[i], ch->z[i], s);
        }
        ch->rowbuf[row] = s;
    }
    return sum_rows(ch, ch->rowbuf);
}

/* tea_leaf_kernel_cuda.cu:494-500: r.z */
double ora_ppcg_calc_zrnorm(ora_chunk *ch) { return dot(ch, ch->r, ch->z); }

/* tea_leaf_ppcg.cuknl:301-313 */
void ora_ppcg_calc_p(ora_chunk *ch, double beta) {
    int h = ch->h;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->p[i] = fma(beta, ch->p[i], ch->z[i]);
        }
}

/* tea_leaf_jacobi.cuknl:5-46 (un lives in its own array here) */
double ora_jacobi_solve(ora_chunk *ch) {
    int h = ch->h;
    const size_t P = (size_t)ch->pitch;
    memcpy(ch->un, ch->u, ch->n2d * sizeof(double));
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row) {
        double s = 0.0;
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            const double *un = ch->un, *kx = ch->kx, *ky = ch->ky;
            double num = fma(kx[i + 1], un[i + 1], ch->u0[i]);
            num = fma(kx[i], un[i - 1], num);
            num = fma(ky[i + P], un[i + P], num);
            num = fma(ky[i], un[i - P], num);
            double den = (1.0 + (kx[i] + kx[i + 1])) + (ky[i] + ky[i + P]);
            ch->u[i] = num / den;
            s += fabs(ch->u[i] - un[i]);
        }
        ch->rowbuf[row] = s;
    }
    return sum_rows(ch, ch->rowbuf);
}

/* tea_leaf_common.cuknl:5-17 */
void ora_finalise(ora_chunk *ch) {
    int h = ch->h;
#pragma omp parallel for schedule(static) if (ch->nx * ch->ny >= ORA_PAR_MIN)
    for (int row = h; row < h + ch->ny; ++row)
        for (int col = h; col < h + ch->nx; ++col) {
            size_t i = IDX(ch, col, row);
            ch->energy1[i] = ch->u[i] / ch->density[i];
        }
}

/* ------------------------------------------------------------------------ */
/* host numerics: tea_leaf_cheby.f90                                        */
/* ------------------------------------------------------------------------ */

/* tqli, tea_leaf_cheby.f90:46-96 (QL with implicit shifts on a symmetric
 * tridiagonal matrix; e holds the sub-diagonal in e[1..n-1] on entry). */
int ora_tqli(double *d, double *e, int n) {
    /* e(:) = eoshift(e(:), 1) */
    for (int i = 0; i < n - 1; ++i) e[i] = e[i + 1];
    if (n > 0) e[n - 1] = 0.0;
    for (int l = 0; l < n; ++l) {
        int iter = 0;
        for (;;) {
            int m;
            for (m = l; m < n - 1; ++m) {
                double dd = fabs(d[m]) + fabs(d[m + 1]);
                if (fabs(e[m]) + dd == dd) break;
            }
            if (m == l) break;
            if (iter == 30) return 1;
            iter++;
            double g = (d[l + 1] - d[l]) / (2.0 * e[l]);
            double r = sqrt(g * g + 1.0);
            g = d[m] - d[l] + e[l] / (g + copysign(fabs(r), g));
            double s = 1.0, c = 1.0, p = 0.0;
            int restart = 0;
            for (int i = m - 1; i >= l; --i) {
                double f = s * e[i];
                double b = c * e[i];
                r = sqrt(f * f + g * g);
                e[i + 1] = r;
                if (r == 0.0) {
                    d[i + 1] -= p;
                    e[m] = 0.0;
                    restart = 1;
                    break;
                }
                s = f / r;
                c = g / r;
                g = d[i + 1] - p;
                r = (d[i] - g) * s + 2.0 * c * b;
                p = s * r;
                d[i + 1] = g + p;
                g = c * r - b;
            }
            if (restart) continue;
            d[l] -= p;
            e[l] = g;
            e[m] = 0.0;
        }
    }
    return 0;
}

/* tea_calc_eigenvalues, tea_leaf_cheby.f90:98-145 */
int ora_calc_eigenvalues(const double *cg_alphas, const double *cg_betas, int n,
                         double *eigmin, double *eigmax) {
    if (n < 1) return 1;
    double *diag = zalloc((size_t)n + 1), *off = zalloc((size_t)n + 1);
    for (int k = 0; k < n; ++k) {
        diag[k] = 1.0 / cg_alphas[k];
        if (k > 0) diag[k] += cg_betas[k - 1] / cg_alphas[k - 1];
        if (k < n - 1) off[k + 1] = sqrt(cg_betas[k]) / cg_alphas[k];
    }
    int info = ora_tqli(diag, off, n);
    if (info == 0) {
        /* ascending sort (the bubble sort of :127-138) */
        for (int a = 1; a < n; ++a) {
            double v = diag[a];
            int b = a - 1;
            while (b >= 0 && diag[b] > v) {
                diag[b + 1] = diag[b];
                b--;
            }
            diag[b + 1] = v;
        }
        *eigmin = diag[0];
        *eigmax = diag[n - 1];
        if (*eigmin < 0.0 || *eigmax < 0.0) info = 1;
    }
    free(diag);
    free(off);
    return info;
}

/* tea_calc_ch_coefs, tea_leaf_cheby.f90:147-174 */
void ora_calc_ch_coefs(double *alphas, double *betas, double eigmin, double eigmax,
                       double *theta_out, int n) {
    double theta = (eigmax + eigmin) / 2.0;
    double delta = (eigmax - eigmin) / 2.0;
    double sigma = theta / delta;
    double rho_old = 1.0 / sigma;
    for (int k = 0; k < n; ++k) {
        double rho_new = 1.0 / (2.0 * sigma - rho_old);
        alphas[k] = rho_new * rho_old;
        betas[k] = 2.0 * rho_new / delta;
        rho_old = rho_new;
    }
    *theta_out = theta;
}

/* ------------------------------------------------------------------------ */
/* solver driver: tea_solve.f90:37-509                                      */
/* ------------------------------------------------------------------------ */

/* tea_leaf_ppcg.f90:174-230 on one chunk */
static void run_ppcg_inner_steps(ora_chunk *ch, double theta) {
    int inner = ch->cfg.ppcg_inner_steps, hd = ch->h;
    halo1(ch, 4, 1);
    if (inner < 0) return;
    ora_ppcg_init_sd_new(ch, theta);
    for (int cur = 1; cur <= inner; cur += hd) {
        halo1(ch, 6, hd);
        for (int be = hd - 1; be >= 0; --be) {
            int st = cur + hd - 1 - be;
            ora_ppcg_inner(ch, st);
            halo1(ch, 6, 1);
            if (st == inner) break;
        }
    }
    ora_ppcg_update_z(ch);
}

static void tea_leaf(ora_chunk *ch, ora_step_result *res) {
    const ora_config *c = &ch->cfg;
    const int use_cg = c->solver == ORA_CG, use_ch = c->solver == ORA_CHEBY,
              use_pp = c->solver == ORA_PPCG, use_jac = c->solver == ORA_JACOBI;
    double old_error, error = 0.0, exact_error = 0.0, initial_residual;
    double rro = 0.0, pw, rrn, alpha, beta;
    int est_itc = 0, cheby_calc_steps = 0, max_cheby_iters = 0, ppcg_inner_iters = 0;
    int ch_switch_check = 0;
    int fields_p = 0, fields_u = 0;
    int n;

    res->switch_n = 0;
    res->est_itc = 0;
    {
        int fl[7] = {1, 0, 1, 0, 0, 0, 0}; /* density, energy1 */
        ora_update_halo(ch, fl, c->halo_depth);
    }
    double rx, ry;
    ora_common_init(ch, ch->dt, &rx, &ry);
    halo1(ch, 4, 1);
    ora_calc_residual(ch);
    initial_residual = ora_calc_2norm(ch, 1);
    old_error = initial_residual;
    initial_residual = sqrt(fabs(initial_residual));

    if (use_cg || use_ch || use_pp) {
        rro = ora_cg_init(ch);
        int fl[7] = {0, 0, 0, 1, 1, 0, 0};
        ora_update_halo(ch, fl, 1);
        fields_p = 1;
    } else if (use_jac) {
        fields_u = 1;
    }

    for (n = 1; n <= c->max_iters; ++n) {
        if (!ch_switch_check) {
            if (cheby_calc_steps > 0) ch_switch_check = 1;
            else if (!ch->first && use_pp && n > 1) ch_switch_check = 1;
            else if (fabs(old_error) <= c->ch_cg_epslim && n >= c->ch_cg_presteps) ch_switch_check = 1;
            else ch_switch_check = 0;
        }
        if ((use_ch || use_pp) && ch_switch_check) {
            if (cheby_calc_steps == 0) {
                max_cheby_iters = c->max_iters - n + 2;
                if (ch->first) {
                    int info = ora_calc_eigenvalues(ch->cg_alphas + 1, ch->cg_betas + 1, n - 1,
                                                    &ch->eigmin, &ch->eigmax);
                    ch->first = 0;
                    if (info != 0) {
                        fprintf(stderr, "tea_leaf: Error in calculating eigenvalues\n");
                        ch->eigmin = ch->eigmax = NAN;
                    }
                    ch->eigmin *= 0.95;
                    ch->eigmax *= 1.05;
                }
                if (use_ch) {
                    ora_calc_ch_coefs(ch->ch_alphas, ch->ch_betas, ch->eigmin, ch->eigmax,
                                      &ch->theta, max_cheby_iters);
                    fields_p = 0;
                    fields_u = 1;
                } else {
                    ora_calc_ch_coefs(ch->ch_alphas, ch->ch_betas, ch->eigmin, ch->eigmax,
                                      &ch->theta, c->ppcg_inner_steps);
                    ora_ppcg_init_constants(ch, ch->ch_alphas, ch->ch_betas, c->ppcg_inner_steps);
                }
                ch->cn = ch->eigmax / ch->eigmin;
                res->switch_n = n;
                res->eigmin = ch->eigmin;
                res->eigmax = ch->eigmax;
                if (use_pp) {
                    /* reinitialise CG with PPCG applied, tea_solve.f90:226-250 */
                    rro = ora_ppcg_init(ch, 2);
                    run_ppcg_inner_steps(ch, ch->theta);
                    ppcg_inner_iters += c->ppcg_inner_steps;
                    rro = ora_ppcg_init(ch, 3);
                    halo1(ch, 5, 1);
                }
            }
            if (use_ch) {
                if (cheby_calc_steps == 0) {
                    /* tea_leaf_cheby_first_step, tea_leaf_cheby.f90:176-220;
                     * its error argument is the caller's old_error */
                    double bb = ora_calc_2norm(ch, 0);
                    ora_cheby_init(ch, ch->ch_alphas, ch->ch_betas, max_cheby_iters, ch->theta);
                    halo1(ch, 4, 1);
                    ora_cheby_iterate(ch, 1);
                    old_error = ora_calc_2norm(ch, 1);
                    double it_alpha = c->eps * bb / (4.0 * old_error);
                    double gamm = (sqrt(ch->cn) - 1.0) / (sqrt(ch->cn) + 1.0);
                    est_itc = (int)lround(log(it_alpha) / (2.0 * log(gamm)));
                    res->est_itc = est_itc;
                    cheby_calc_steps = 1;
                } else {
                    ora_cheby_iterate(ch, cheby_calc_steps);
                    if (n >= est_itc && n % 10 == 0) error = ora_calc_2norm(ch, 1);
                }
            } else if (use_pp) {
                pw = ora_cg_calc_w(ch);
                ora_ppcg_store_r(ch);
                rro = ora_ppcg_calc_zrnorm(ch);
                alpha = rro / pw;
                (void)ora_cg_calc_ur(ch, alpha);
                run_ppcg_inner_steps(ch, ch->theta);
                ppcg_inner_iters += c->ppcg_inner_steps;
                rrn = ora_ppcg_calc_rrn(ch);
                beta = rrn / rro;
                ora_ppcg_calc_p(ch, beta);
                error = rrn;
                rro = rrn;
            }
            cheby_calc_steps++;
        } else if (use_cg || use_ch || use_pp) {
            fields_p = 1;
            pw = ora_cg_calc_w(ch);
            alpha = rro / pw;
            ch->cg_alphas[n] = alpha;
            rrn = ora_cg_calc_ur(ch, alpha);
            beta = rrn / rro;
            ch->cg_betas[n] = beta;
            ora_cg_calc_p(ch, beta);
            error = rrn;
            rro = rrn;
        } else if (use_jac) {
            error = ora_jacobi_solve(ch);
        }
        {
            int fl[7] = {0, 0, 0, fields_u, fields_p, 0, 0};
            ora_update_halo(ch, fl, 1);
        }
        error = sqrt(fabs(error));
        if (fabs(error) < c->eps * initial_residual) break;
        old_error = error;
    }

    if (c->check_result) {
        halo1(ch, 4, 1);
        ora_calc_residual(ch);
        exact_error = sqrt(ora_calc_2norm(ch, 1));
    }
    res->initial_residual = initial_residual;
    res->error = error;
    res->error_ratio = error / initial_residual;
    res->exact_error_ratio = c->check_result ? exact_error / initial_residual : 0.0;
    res->iterations = n - 1;
    res->ppcg_inner_iters = ppcg_inner_iters;
    ora_finalise(ch);
    halo1(ch, 3, 1);
}

int ora_start(ora_chunk *ch, ora_step_result *s0) {
    ch->time = 0.0;
    ch->step = 0;
    ch->dt = ch->cfg.dtinit;
    ch->complete = 0;
    initialise_chunk(ch);
    generate_chunk(ch);
    int fl[7] = {1, 1, 1, 0, 0, 0, 0};
    ora_update_halo(ch, fl, ch->h);
    set_field(ch);
    memset(s0, 0, sizeof *s0);
    s0->step = 0;
    s0->has_summary = 1;
    ora_field_summary(ch, &s0->vol, &s0->mass, &s0->ie, &s0->temp);
    return 0;
}

int ora_step(ora_chunk *ch, ora_step_result *res) {
    memset(res, 0, sizeof *res);
    ch->step += 1;
    /* timestep.f90 + calc_dt.f90: dt = min(dt, dtinit) */
    if (ch->cfg.dtinit <= ch->dt) ch->dt = ch->cfg.dtinit;
    res->step = ch->step;
    res->time = ch->time;
    res->dt = ch->dt;
    tea_leaf(ch, res);
    ch->time += ch->dt;
    int sf = ch->cfg.summary_frequency;
    if (sf != 0 && ch->step % sf == 0) {
        res->has_summary = 1;
        ora_field_summary(ch, &res->vol, &res->mass, &res->ie, &res->temp);
    }
    if (ch->time + G_SMALL > ch->cfg.end_time || ch->step >= ch->cfg.end_step) {
        ch->complete = 1;
        res->has_summary = 1;
        ora_field_summary(ch, &res->vol, &res->mass, &res->ie, &res->temp);
        return 1;
    }
    return 0;
}
