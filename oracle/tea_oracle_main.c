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

static void print_step(const ora_step_result *r, double wall) {
    printf("{\"kind\": \"step\", \"step\": %d, \"iterations\": %d, \"ppcg_inner\": %d, "
           "\"error_ratio\": %.17g, \"switch_n\": %d, \"est_itc\": %d, \"wall\": %.6f",
           r->step, r->iterations, r->ppcg_inner_iters, r->error_ratio, r->switch_n,
           r->est_itc, wall);
    if (r->has_summary)
        printf(", \"vol\": %.17g, \"mass\": %.17g, \"ie\": %.17g, \"temp\": %.17g", r->vol,
               r->mass, r->ie, r->temp);
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
