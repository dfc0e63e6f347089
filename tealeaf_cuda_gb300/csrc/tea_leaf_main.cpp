// tea_leaf_main.cpp -- the `tea_leaf` executable: reads a deck (./tea.in by
// default), writes tea.out, echoes the log like the reference program.
//   tea_leaf [deck] [--out FILE] [--legacy-abi] [--max-steps N] [--quiet] [--model FILE]
// --model names the network of `tl_warm_start learned` (a TLWS0001 file).
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <string>

#include "../../include/tealeaf_capi.h"

int main(int argc, char **argv) {
    const char *deck = "tea.in";
    const char *out = "tea.out";
    tl_run_options_t o;
    memset(&o, 0, sizeof o);
    o.echo = 1;
    for (int i = 1; i < argc; ++i) {
        if (!strcmp(argv[i], "--out") && i + 1 < argc) out = argv[++i];
        else if (!strcmp(argv[i], "--legacy-abi")) o.legacy_abi = 1;
        else if (!strcmp(argv[i], "--max-steps") && i + 1 < argc) o.max_steps = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--quiet")) o.echo = 0;
        else if (!strcmp(argv[i], "--model") && i + 1 < argc) o.model_path = argv[++i];
        else deck = argv[i];
    }
    FILE *f = fopen(deck, "rb");
    if (!f) {
        fprintf(stderr, "tea_leaf: cannot open %s\n", deck);
        return 2;
    }
    std::string text;
    char buf[4096];
    size_t n;
    while ((n = fread(buf, 1, sizeof buf, f)) > 0) text.append(buf, n);
    fclose(f);
    o.out_path = out;
    tl_run_result_t r;
    int rc = tl_run_deck(text.c_str(), &o, &r);
    if (rc < 0) {
        fprintf(stderr, "tea_leaf: failed (%d): %s\n", rc, tl_last_error());
        return 1;
    }
    return 0;
}
