/*
 * og_cli.c -- command-line front end of the CPU oracle (test infrastructure).
 *
 *   og_cli <graph> <src> <dst> [--rule level|fifo] [--precheck] [--order waves|heap|dfs]
 *          [--eps f] [--target f] [--capacity n] [--shift s] [--buckets b] [--threads t]
 *          [--brute]
 *
 * Prints the result fields one per line as "key value" for scripts.
 */
#include "oracle.h"

#include <stdio.h>
#include <stdlib.h>
#include <string.h>

int main(int argc, char **argv)
{
    if (argc < 4) {
        fprintf(stderr, "usage: %s <graph> <src> <dst> [options]\n", argv[0]);
        return 1;
    }
    og_graph g;
    int rc = og_load(argv[1], &g);
    if (rc) { fprintf(stderr, "cannot load %s (%d)\n", argv[1], rc); return 1; }
    int src = atoi(argv[2]), dst = atoi(argv[3]);
    og_opts o;
    og_default_opts(&o);
    int brute = 0;
    for (int i = 4; i < argc; i++) {
        const char *a = argv[i];
        const char *v = (i + 1 < argc) ? argv[i + 1] : NULL;
        if (!strcmp(a, "--rule") && v) { o.bfs_rule = !strcmp(v, "fifo") ? OG_BFS_FIFO : OG_BFS_LEVEL; i++; }
        else if (!strcmp(a, "--precheck")) o.precheck = 1;
        else if (!strcmp(a, "--order") && v) {
            o.order = !strcmp(v, "heap") ? OG_ORDER_HEAP : !strcmp(v, "dfs") ? OG_ORDER_DFS : OG_ORDER_WAVES;
            i++;
        }
        else if (!strcmp(a, "--eps") && v) { o.eps = atof(v); i++; }
        else if (!strcmp(a, "--target") && v) { o.target_width = atof(v); i++; }
        else if (!strcmp(a, "--capacity") && v) { o.capacity = strtoull(v, NULL, 10); i++; }
        else if (!strcmp(a, "--shift") && v) { o.bucket_shift = atoi(v); i++; }
        else if (!strcmp(a, "--buckets") && v) { o.n_buckets = atoi(v); i++; }
        else if (!strcmp(a, "--threads") && v) { o.threads = atoi(v); i++; }
        else if (!strcmp(a, "--max_nodes") && v) { o.max_nodes = strtoull(v, NULL, 10); i++; }
        else if (!strcmp(a, "--brute")) brute = 1;
    }
    printf("N %d\nE %d\n", g.n_nodes, g.n_edges);
    if (brute) {
        printf("brute %.20f\n", og_brute(&g, src, dst));
    } else {
        og_result r;
        og_run(&g, src, dst, &o, &r);
        printf("R %.20f\nesp %.6e\npaths %llu\nnodes %llu\nleaves %llu\ndead %llu\ntruncated %llu\n"
               "spilled %llu\npruned %llu\nwaves %llu\nmax_wave %llu\nmax_queued %llu\nstatus %d\n"
               "seconds %.6f\n",
               r.R, r.esp, (unsigned long long)r.paths, (unsigned long long)r.nodes,
               (unsigned long long)r.leaves, (unsigned long long)r.dead, (unsigned long long)r.truncated,
               (unsigned long long)r.spilled, (unsigned long long)r.pruned, (unsigned long long)r.waves,
               (unsigned long long)r.max_wave, (unsigned long long)r.max_queued, r.status, r.seconds);
    }
    og_free_graph(&g);
    return 0;
}
