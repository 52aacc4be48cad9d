/*
 * oracle.h -- CPU oracle for two-terminal network reliability by path
 * decomposition.
 *
 * TEST INFRASTRUCTURE ONLY.  Nothing in the product (the CUDA engine, the
 * C ABI in include/nr.h, the CLI) links or calls this code.  Only tests/,
 * __graft_entry__.smoke() and bench.py's CPU-baseline leg use it, as the
 * checker and as the timed CPU port of the reference algorithm.
 *
 * What it restates (paths relative to the fmalazemi/relaibilityGPU tree):
 *   graph file + edge ids ..... workingPad/graph.h:46-145 (first-seen (min,max)
 *                               pair order while scanning nodes in order)
 *   initial mask .............. workingPad/main.cu:717-748
 *   BFS, parent rule "level" .. workingPad/device_code.cuh:80-194 (bitmask
 *                               frontier scanned in ascending node order, so
 *                               parent[v] = smallest frontier node with a
 *                               not-down arc to v)
 *   BFS, parent rule "fifo" ... seq/seq.cpp:311-351 (FIFO queue, first
 *                               discoverer, early exit at t)
 *   branching ................. workingPad/main.cu:114-283 and
 *                               seq/seq.cpp:539-578 (child k = first k-1
 *                               UNKNOWN path edges up, k-th down, src side
 *                               first; all-up mass -> R)
 *   K-terminal ................ the same decomposition over the BFS tree that joins
 *                               every terminal to src (the union of the parent
 *                               paths), its edges in BFS order; the reference only
 *                               stubs a target set (parallel/Rel_16M.cu:43)
 *   fork branching ............ workingPad/main.cu:303-430 with :550-565
 *                               (FORK_BEST_EDGE) and seq/seq_best.cpp:358-389:
 *                               a path of up edges puts the whole mass in R;
 *                               else the UNKNOWN edge of the optimistic path
 *                               with the largest p (ties: the one nearest
 *                               dst) gives two children, down and up
 *   counts .................... workingPad/main.cu:533-534 (every pop is a
 *                               node), :251 and :262 (overflow spills and
 *                               leaves are paths); seq/seq.cpp:551-561
 *                               (pre-push connectivity check)
 *   eps truncation ............ workingPad/main.cu:537-543
 *   max-mass order ............ seq/seq.cpp:49-197
 *   brute force ............... 2^E state enumeration (definition of R)
 *
 * Masses are FP64 products in path order (not log sums) and every sum is
 * compensated (two-sum), so R is accurate to ~1e-16 relative.
 */
#ifndef NR_ORACLE_H
#define NR_ORACLE_H

#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

typedef struct og_graph {
    int32_t n_nodes;
    int32_t n_edges;
    int32_t n_arcs;
    const int32_t *row_ptr;   /* n_nodes + 1 */
    const int32_t *col_idx;   /* n_arcs */
    const int32_t *edge_id;   /* n_arcs */
    const double  *edge_p;    /* n_edges */
} og_graph;

enum { OG_BFS_LEVEL = 0, OG_BFS_FIFO = 1 };
enum { OG_ORDER_WAVES = 0, OG_ORDER_HEAP = 1, OG_ORDER_DFS = 2 };
enum { OG_BRANCH_PATH = 0, OG_BRANCH_FORK = 1 };

typedef struct og_opts {
    int32_t  bfs_rule;      /* OG_BFS_LEVEL (GPU engine, main.cu) or OG_BFS_FIFO (seq.cpp) */
    int32_t  precheck;      /* 1: drop disconnected children before queueing (seq.cpp) */
    int32_t  order;         /* OG_ORDER_* */
    int32_t  bucket_shift;  /* waves: 2^shift mass buckets per octave; < 0: one bucket */
    int32_t  n_buckets;     /* waves: number of buckets (the last one takes all smaller masses) */
    int32_t  threads;       /* waves: worker threads (>= 1) */
    double   eps;           /* popped mass < eps goes to ESP unexpanded; 0 disables */
    double   target_width;  /* waves/heap: stop once ESP + queued mass <= target; 0 disables */
    uint64_t capacity;      /* queued-item limit, overflow spills to ESP; 0 = unlimited */
    uint64_t max_nodes;     /* stop after about this many pops (timing samples); 0 = none */
    int32_t  branching;     /* OG_BRANCH_PATH (disjoint path children) or OG_BRANCH_FORK */
    int32_t  n_terminals;   /* K-terminal: > 0 with `terminals` below; src is terminals[0] */
    const int32_t *terminals;
    int32_t  branch_order;  /* path branching, the order the path's UNKNOWN edges are branched in:
                               OG_BORDER_SRC (the reference), _DST, _P_ASC, _P_DESC */
} og_opts;

enum { OG_BORDER_SRC = 0, OG_BORDER_DST = 1, OG_BORDER_P_ASC = 2, OG_BORDER_P_DESC = 3 };

typedef struct og_result {
    double   R;             /* reliability found (sum of all-up leaf masses) */
    double   esp;           /* spilled + eps-truncated + still-queued mass */
    double   esp_spilled;
    double   esp_truncated;
    double   queued_mass;
    uint64_t paths;         /* leaves + overflow spills (main.cu:251,262) */
    uint64_t nodes;         /* pops, including dead ends and truncated items */
    uint64_t leaves;
    uint64_t dead;          /* pops whose optimistic BFS fails */
    uint64_t truncated;     /* pops below eps */
    uint64_t spilled;       /* children that did not fit */
    uint64_t pruned;        /* children dropped by the pre-push check */
    uint64_t pushes;
    uint64_t waves;
    uint64_t max_wave;
    uint64_t max_queued;
    uint64_t queued;        /* items left in the queue at the end */
    int32_t  status;        /* 0 done, 1 target width reached, 2 max_nodes reached, <0 error */
    double   seconds;
} og_result;

/* Parse the reference graph file format: "N E [U|D]" then N lines "deg (nbr p)*".
 * Arrays are malloc'd; release with og_free_graph. Returns 0 or a negative error. */
int  og_load(const char *path, og_graph *g);
void og_free_graph(og_graph *g);

void og_default_opts(og_opts *o);
int  og_run(const og_graph *g, int src, int dst, const og_opts *o, og_result *r);

/* Solve n instances, one per worker thread at a time (wave schedule, single-
 * threaded per instance, storage reused across instances). */
int  og_run_batch(int n, const og_graph *graphs, const int32_t *srcs, const int32_t *dsts,
                  const og_opts *o, og_result *results, int threads);

/* Exact R by enumerating the 2^k states of the k edges with 0 < p < 1.
 * n_nodes <= 64, k <= 30. Returns a negative number on bad input. */
double og_brute(const og_graph *g, int src, int dst);

/* The same for K-terminal reliability: every node of `terminals` connected to terminals[0]. */
double og_brute_k(const og_graph *g, const int32_t *terminals, int n_terminals);

/* The ceiling of queue orders (an experiment, not the reference's method).
 * Popping a subproblem takes its "gain" out of the width ESP + queued mass: the all-up
 * leaf mass of a live subproblem, the whole mass of a dead end.  For a branching rule
 * (path branching with o->branch_order; eps 0, no capacity), every order reaches
 * width <= target only once the gains of the popped subproblems add up to >= 1 - target,
 * so no order needs fewer pops than the smallest k for which the k largest gains of the
 * whole decomposition tree reach 1 - target (min_pops).  Those gains are found by
 * max-mass best-first search: a gain never exceeds its subproblem's mass and masses
 * shrink down the tree, so once the k-th largest gain seen is >= the largest queued
 * mass, no unseen subproblem can be among the k largest.  Breadth-first waves reach
 * the largest gain any schedule can after h parallel steps (the first h levels of the
 * tree hold every subproblem a height-h subtree can), so bf_waves is the fewest steps
 * any schedule needs.  plain_pops: max-mass (heap) order; bf_pops: breadth-first.
 * status 0, or 2 if `budget` pops ran out before min_pops was certain. */
typedef struct og_bound {
    uint64_t plain_pops, min_pops, bf_pops, bf_waves, explored;
    int32_t  status;
    int32_t  pad;
} og_bound;
int og_order_bound(const og_graph *g, int src, int dst, const og_opts *o, uint64_t budget, og_bound *out);

/* Bucket index used by the wave schedule (shared definition with the engine). */
int og_bucket(double mass, int shift, int n_buckets);

#ifdef __cplusplus
}
#endif
#endif
