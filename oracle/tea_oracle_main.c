/*
 * tea_oracle_main.c -- command-line front end of the CPU oracle (test
 * infrastructure).  Runs a tea.in deck through the oracle and prints one JSON
 * object per line: a "step" record per timestep and a final "run" record.
 *
 *   tea_oracle <deck> [--max-steps N]
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

static void print_step(const ora_step_result *r, double wall) {
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
    printf("}\n");
    fflush(stdout);
}

int main(int argc, char **argv) {
    if (argc < 2) {
        fprintf(stderr, "usage: %s <deck> [--max-steps N]\n", argv[0]);
        return 2;
    }
    int max_steps = -1;
    for (int i = 2; i < argc; ++i)
        if (!strcmp(argv[i], "--max-steps") && i + 1 < argc) max_steps = atoi(argv[++i]);
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
    ora_step_result r;
    ora_start(ch, &r);
    print_step(&r, 0.0);
    double t0 = now();
    long total_its = 0;
    int steps = 0;
    for (;;) {
        int done = ora_step(ch, &r);
        steps++;
        total_its += r.iterations;
        print_step(&r, now() - t0);
        if (done || (max_steps > 0 && steps >= max_steps)) break;
    }
    double wall = now() - t0;
    printf("{\"kind\": \"run\", \"steps\": %d, \"total_iterations\": %ld, \"wall\": %.6f, "
           "\"threads\": %d, \"cells\": %ld}\n",
           steps, total_its, wall, ora_num_threads(), (long)cfg.x_cells * cfg.y_cells);
    ora_chunk_free(ch);
    free(text);
    return 0;
}
