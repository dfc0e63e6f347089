/*
 * tea_oracle_main.c -- command-line front end of the CPU oracle (test
 * infrastructure).  Runs a tea.in deck through the oracle and prints one JSON
 * object per line: a "step" record per timestep and a final "run" record.
 *
 *   tea_oracle <deck> [--max-steps N] [--u-samples S]
 *
 * --u-samples S adds to every step record the solution u at an S x S lattice
 * of interior cells (cell centres of an even S x S partition of the grid, row
 * by row), so that a solve on another machine can be compared with this one
 * point by point without storing whole fields.
 */
#include "tea_oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>
#include <math.h>
#include <time.h>

static char *slurp(const char *path) {
    FILE *f = fopen(path, "rb");
    if (!f) return NULL;
    fseek(f, 0, SEEK_END);
    long n = ftell(f);
    fseek(f, 0, SEEK_SET);
    char *buf = (char *)malloc((size_t)n + 1);
    if (!buf) { fclose(f); return NULL; }
    size_t got = fread(buf, 1, (size_t)n, f);
    buf[got] = '\0';
    fclose(f);
    return buf;
}

static double now(void) {
    struct timespec ts;
    clock_gettime(CLOCK_MONOTONIC, &ts);
    return (double)ts.tv_sec + 1e-9 * (double)ts.tv_nsec;
}

/* a double as a JSON number; NaN and infinities in the spelling Python's
 * json module reads */
static void num(const char *key, double v) {
    if (isnan(v)) printf(", \"%s\": NaN", key);
    else if (isinf(v)) printf(", \"%s\": %sInfinity", key, v < 0 ? "-" : "");
    else printf(", \"%s\": %.17g", key, v);
}

/* the lattice of --u-samples: S points per axis at the centres of an even
 * partition of n cells, as 0-based interior indices */
static int sample_index(int k, int s, int n) {
    return (int)(((2L * k + 1) * (long)n) / (2L * s));
}

static void print_step(const ora_step_result *r, double wall, const ora_chunk *ch,
                       const ora_config *cfg, int u_samples, double *ubuf) {
    printf("{\"kind\": \"step\", \"step\": %d, \"iterations\": %d, \"ppcg_inner\": %d, "
           "\"switch_n\": %d, \"est_itc\": %d, \"wall\": %.6f",
           r->step, r->iterations, r->ppcg_inner_iters, r->switch_n, r->est_itc, wall);
    num("error_ratio", r->error_ratio);
    if (r->has_summary) {
        num("vol", r->vol);
        num("mass", r->mass);
        num("ie", r->ie);
        num("temp", r->temp);
    }
    if (u_samples > 0 && ubuf) {
        ora_get_field(ch, ORA_F_U, ubuf);
        const int h = cfg->halo_depth, pitch = ora_field_pitch(ch);
        printf(", \"u_samples\": [");
        for (int j = 0; j < u_samples; ++j)
            for (int i = 0; i < u_samples; ++i) {
                const int y = h + sample_index(j, u_samples, cfg->y_cells);
                const int x = h + sample_index(i, u_samples, cfg->x_cells);
                printf("%s%.17g", (i | j) ? ", " : "", ubuf[(size_t)y * pitch + x]);
            }
        printf("]");
    }
    printf("}\n");
    fflush(stdout);
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s <deck> [--max-steps N]\n", argv[0]);
        return 2;
    }
    int max_steps = -1, u_samples = 0;
    for (int i = 2; i < argc; ++i) {
        if (!strcmp(argv[i], "--max-steps") && i + 1 < argc) max_steps = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--u-samples") && i + 1 < argc) u_samples = atoi(argv[++i]);
    }
    char *text = slurp(argv[1]);
    if (!text) {
        fprintf(stderr, "cannot read %s\n", argv[1]);
        return 2;
    }
    ora_config cfg;
    char err[256];
    if (ora_parse_deck(text, &cfg, err, sizeof err) != 0) {
        fprintf(stderr, "deck error: %s\n", err);
        return 3;
    }
    ora_chunk *ch = ora_chunk_new(&cfg);
    if (!ch) return 4;
    double *ubuf = NULL;
    if (u_samples > 0) {
        const int h = cfg.halo_depth;
        ubuf = (double *)malloc((size_t)(cfg.y_cells + 2 * h) * ora_field_pitch(ch) * sizeof(double));
        if (!ubuf) return 4;
    }
    ora_step_result r;
    ora_start(ch, &r);
    print_step(&r, 0.0, ch, &cfg, u_samples, ubuf);
    double t0 = now();
    long total_its = 0;
    int steps = 0;
    for (;;) {
        int done = ora_step(ch, &r);
        steps++;
        total_its += r.iterations;
        print_step(&r, now() - t0, ch, &cfg, u_samples, ubuf);
        if (done || (max_steps > 0 && steps >= max_steps)) break;
    }
    free(ubuf);
    double wall = now() - t0;
    printf("{\"kind\": \"run\", \"steps\": %d, \"total_iterations\": %ld, \"wall\": %.6f, "
           "\"threads\": %d, \"cells\": %ld}\n",
           steps, total_its, wall, ora_num_threads(), (long)cfg.x_cells * cfg.y_cells);
    ora_chunk_free(ch);
    free(text);
    return 0;
}
