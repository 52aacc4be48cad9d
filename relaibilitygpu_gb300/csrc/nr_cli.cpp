// nr_cli.cpp -- `network_reliability`, a drop-in for the reference program
// (workingPad/main.cu:753-790 arguments, :1037-1056 result block).
//
//   network_reliability <graph_file> <src> <dst> [--truncation_eps f]
//       [--queue_capacity n] [--thresh_high f] [--thresh_low f]
//       [--target_width f] [--order auto|waves|maxmass|learned] [--fork] [--device d]
//
// --fork selects the reference's FORK_BEST_EDGE branching (main.cu:21, :550-565).
//
// --thresh_high / --thresh_low are accepted and ignored, as in the reference
// (parsed at main.cu:783-786, never used).  Unknown flags are ignored too.
// Unlike the reference, src and dst are range-checked.
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

#include "nr.h"

static void usage(const char *prog)
{
    fprintf(stderr,
            "Usage: %s <graph_file> <src> <dst> [options]\n"
            "Options:\n"
            "  --truncation_eps <float>   Truncation epsilon (default 1e-15)\n"
            "  --queue_capacity <int>     Per-queue capacity  (default %d)\n"
            "  --thresh_high <float>      High-priority log-prob threshold\n"
            "  --thresh_low  <float>      Low-priority  log-prob threshold\n"
            "  --target_width <float>     Stop once ESP + queued mass <= target (default: off)\n"
            "  --order <auto|waves|maxmass|learned>\n"
            "  --fork                     Fork on the most reliable path edge (FORK_BEST_EDGE)\n"
            "  --device <int>             CUDA device (default 0)\n",
            prog, 1 << 20);
}

int main(int argc, char **argv)
{
    if (argc < 4) {
        usage(argv[0]);
        return 1;
    }
    const char *path = argv[1];
    const int src = atoi(argv[2]);
    const int dst = atoi(argv[3]);
    nr_options opt;
    nr_options_default(&opt);
    opt.truncation_eps = 1e-15;   // reference CLI default (common.h:34)
    unsigned long long capacity = 1u << 20;
    for (int i = 4; i < argc; ++i) {
        const bool has = i + 1 < argc;
        if (!strcmp(argv[i], "--truncation_eps") && has) opt.truncation_eps = atof(argv[++i]);
        else if (!strcmp(argv[i], "--queue_capacity") && has) capacity = strtoull(argv[++i], nullptr, 10);
        else if (!strcmp(argv[i], "--thresh_high") && has) ++i;
        else if (!strcmp(argv[i], "--thresh_low") && has) ++i;
        else if (!strcmp(argv[i], "--target_width") && has) opt.target_width = atof(argv[++i]);
        else if (!strcmp(argv[i], "--device") && has) opt.device = atoi(argv[++i]);
        else if (!strcmp(argv[i], "--fork")) opt.branching = NR_BRANCH_FORK;
        else if (!strcmp(argv[i], "--order") && has) {
            const char *o = argv[++i];
            opt.order = !strcmp(o, "waves") ? NR_ORDER_WAVES
                        : !strcmp(o, "maxmass") ? NR_ORDER_MAXMASS
                        : !strcmp(o, "learned") ? NR_ORDER_LEARNED
                                                : NR_ORDER_AUTO;
        }
    }
    nr_graph g;
    int rc = nr_graph_load(path, &g);
    if (rc != NR_OK) {
        fprintf(stderr, "Cannot load %s: %s\n", path, nr_status_string(rc));
        return 1;
    }
    const int words = (2 * g.n_edges + 31) / 32;
    printf("Graph loaded: N=%d  E=%d  mask_words=%d  src=%d  dst=%d\n", g.n_nodes, g.n_edges, words, src, dst);
    nr_result res;
    rc = nr_reliability(&g, src, dst, capacity, &opt, &res);
    if (rc != NR_OK) {
        fprintf(stderr, "network_reliability: %s\n", nr_status_string(rc));
        nr_graph_free(&g);
        return 1;
    }
    printf("Launch config: %d blocks x %d threads, %d B per queued subproblem\n", res.grid_blocks,
           res.block_threads, res.item_bytes);
    char buf[4096];
    nr_format_result(&res, buf, sizeof(buf));
    fputs(buf, stdout);
    nr_graph_free(&g);
    return 0;
}
