/*
 * nr.h -- C ABI of the GB300 two-terminal network reliability engine.
 *
 * The engine computes R(G; s, t), the probability that terminal t can be
 * reached from terminal s when every edge works independently with its own
 * probability, by the path-decomposition (factoring) method of
 * fmalazemi/relaibilityGPU.  It returns the same result block as the
 * reference's `network_reliability` program (workingPad/main.cu:1037-1056):
 * R, R + ESP, ESP, the truncation bound, paths enumerated, nodes processed,
 * kernel iterations and the largest queue.
 *
 * The reference has no library interface: its only caller is its own
 * command-line driver (workingPad/main.cu:795-1072).  Each entry point below
 * names the reference code it stands in for.  Plain C types only; no CUDA or
 * torch type appears in a signature.
 *
 * Status codes: every entry point returns NR_OK (0) or a negative NR_ERR_*;
 * nothing calls exit() (the reference exits on errors, common.h:39-46,
 * graph.h:49-69).  Calls on one nr_context are not re-entrant; separate
 * contexts may be used from separate threads.
 */
#ifndef NR_H
#define NR_H

#include <stddef.h>
#include <stdint.h>

#ifdef __cplusplus
extern "C" {
#endif

#define NR_ABI_VERSION 2

/* status codes */
enum {
    NR_OK              = 0,
    NR_ERR_INVALID     = -1,   /* bad argument (terminal out of range, null pointer, ...) */
    NR_ERR_IO          = -2,   /* graph file missing or unreadable */
    NR_ERR_PARSE       = -3,   /* malformed graph file */
    NR_ERR_UNSUPPORTED = -4,   /* graph outside the engine's limits */
    NR_ERR_CUDA        = -5,   /* CUDA runtime error (no device, launch failure, ...) */
    NR_ERR_NOMEM       = -6,   /* device or host allocation failed */
    NR_ERR_TIMEOUT     = -7,   /* a bounded device-side wait gave up */
    NR_ERR_INTERNAL    = -8    /* a device-side consistency check failed */
};

/* edge states in a subproblem mask: 2 bits per edge id, edge e at word e/16,
 * bits 2*(e%16)..+1 (workingPad/common.h:22-24). */
enum { NR_EDGE_DOWN = 0, NR_EDGE_UP = 1, NR_EDGE_UNKNOWN = 3 };

/* Graph in the reference loader's host form (workingPad/graph.h:12-27):
 * CSR arcs in adjacency-list order, an edge id per arc, a probability per
 * edge id.  Undirected graphs list every edge in both endpoint lists with
 * the same id.  The caller owns all arrays. */
typedef struct nr_graph {
    int32_t        n_nodes;
    int32_t        n_edges;     /* distinct edge ids 0..n_edges-1 */
    int32_t        n_arcs;      /* CSR entries */
    const int32_t *row_ptr;     /* [n_nodes + 1] */
    const int32_t *col_idx;     /* [n_arcs] */
    const int32_t *edge_id;     /* [n_arcs] */
    const double  *edge_p;      /* [n_edges], FP64 */
} nr_graph;

/* queue order */
enum {
    NR_ORDER_AUTO    = 0,   /* waves for exhaustive runs, max-mass buckets when a target width is set */
    NR_ORDER_WAVES   = 1,   /* breadth-first waves, as the reference's ping-pong queue (main.cu:963-1008);
                               with a target width, one bucket whatever bucket_shift says */
    NR_ORDER_MAXMASS = 2,   /* bucketed max-mass priority queue */
    NR_ORDER_LEARNED = 3    /* bucket key and branch order from the learned scorer (never mass) */
};

/* kernel of the warp engine (batches and small truncated runs, n <= 32) */
enum {
    NR_SMALL_AUTO = 0,      /* one lane per subproblem where it applies (undirected simple graphs of
                               <= 16 nodes, path branching, plain order; <= 32 nodes in breadth-first
                               waves with two instances a warp; and the whole-GPU wave engine for
                               <= 32 nodes), lane groups elsewhere */
    NR_SMALL_GROUP = 1,     /* a lane group (one lane per node) per subproblem for every instance,
                               in the warp engine and in the whole-GPU engine for <= 32 nodes */
    NR_SMALL_LANE1 = 2      /* where one lane per subproblem applies, one instance per warp (with one
                               bucket the default gives a warp two instances, interleaving their steps) */
};
enum { NR_KERNEL_GROUP = 1, NR_KERNEL_LANE = 2, NR_KERNEL_LANE2 = 3,
       NR_KERNEL_BLOCK = 4 /* handed over by the two-slot kernel: one instance a block */ };

/* branching of a subproblem whose optimistic BFS finds a path */
enum {
    NR_BRANCH_PATH = 0,     /* one disjoint child per UNKNOWN path edge (main.cu:114-283, the default) */
    NR_BRANCH_FORK = 1      /* a path of up edges puts the mass in R; else fork on the optimistic path's
                               UNKNOWN edge with the largest p, down and up (main.cu:303-430 with
                               :550-565, FORK_BEST_EDGE); not with NR_ORDER_LEARNED */
};

/* branch order: the order in which a path's UNKNOWN edges are branched (child k = the
 * first k-1 of them in this order up, the k-th down).  Every order is a disjoint
 * decomposition, so exhaustive R is the same; the tree, hence the work to a target
 * width, is not. */
enum {
    NR_BORDER_SRC     = 0,  /* src side first (main.cu:114-283, seq.cpp:539-568; the default) */
    NR_BORDER_DST     = 1,  /* dst side first */
    NR_BORDER_P_ASC   = 2,  /* least reliable edge first (ties: path order, src side first) */
    NR_BORDER_P_DESC  = 3,  /* most reliable edge first (ties: path order) */
    NR_BORDER_LEARNED = 4   /* by the learned scorer (nr_context_set_model): edge e first when
                               (1 - p_e) x (1 - r(e)) is largest, r(e) the scorer's residual
                               reliability of the subproblem with e down -- a likely and critical
                               failure first; ties: path order.  The warp engine (n <= 32) with a
                               target width or a max-mass / learned order, and the bucketed
                               whole-GPU queue (n > 32, max-mass order), only */
};

typedef struct nr_options {
    double   truncation_eps;  /* popped mass below eps goes to ESP (main.cu:537-543); 0 = off.
                                 The reference CLI default is 1e-15. */
    double   target_width;    /* stop once ESP + queued mass <= target; 0 = run to empty queue */
    int32_t  order;           /* NR_ORDER_* */
    int32_t  bucket_shift;    /* max-mass order: 2^shift buckets per factor of two in mass; -1 = one
                                 bucket (breadth-first waves, still stopped by target_width) */
    int32_t  n_buckets;       /* max-mass order: bucket count; the last takes all smaller masses */
    int32_t  device;          /* CUDA device ordinal */
    int32_t  blocks_per_sm;   /* 0 = occupancy maximum */
    int32_t  warps_per_block; /* 0 = engine default */
    double   timeout_ms;      /* device-side waits give up after this long without progress; 0 = 60 s */
    int32_t  verbose;         /* 1: print the reference's preamble lines on stdout */
    int32_t  test_fault;      /* tests of the failure paths only; 0 = off (always, in use).
                                 1: block 0 of the cooperative whole-GPU launch leaves before its
                                 first grid barrier, so the other blocks' bounded waits run out
                                 (NR_ERR_TIMEOUT after timeout_ms);
                                 2: the lane kernels' step bound is one step, so their
                                 self-check ends the instance (NR_ERR_INTERNAL).
                                 Nothing faults: every wait and check returns a status. */
    uint64_t max_nodes;       /* per-instance pop budget for the warp engine; truncated runs stop
                                 there with a valid R <= true <= R + ESP bracket, exhaustive runs
                                 hand the instance to the whole-GPU engine; 0 = engine default */
    int32_t  pages_per_warp;  /* warp engine: queue pages of 32 subproblems per warp when capacity is 0
                                 (0 = 512) */
    int32_t  branching;       /* NR_BRANCH_* */
    int32_t  small_kernel;    /* NR_SMALL_*: the warp engine's kernel */
    int32_t  lane_slots;      /* one lane per subproblem, one bucket: instances a warp carries (2 or 4;
                                 0 = the default, 2: on 4096 K15 instances 4 slots leave too few warps
                                 per SM to hide the steps' latency, 0.096 against 0.060 ms) */
    int32_t  branch_order;    /* NR_BORDER_*: path branching only; two-terminal runs (K-terminal runs
                                 take NR_BORDER_SRC) */
    int32_t  handover_pages;  /* breadth-first waves, two instances a warp: an instance whose next wave
                                 holds more than this many pages of 32 subproblems runs again from its
                                 root on a block of warps (the block kernel), with the same schedule and
                                 results; 0 = the default (8 pages), -1 = never */
} nr_options;

typedef struct nr_result {
    double   R;                 /* reliability found: sum of all-up path masses */
    double   R_plus_esp;        /* upper bound */
    double   esp;               /* ESP: eps-truncated + spilled + still-queued mass */
    double   trunc_bound;       /* esp / R when R > 0 (main.cu:1047-1048) */
    uint64_t paths;             /* all-up leaves + queue-overflow spills (main.cu:251,262) */
    uint64_t nodes;             /* subproblems popped, dead ends and truncated ones included (main.cu:533) */
    uint64_t leaves;
    uint64_t dead_ends;
    uint64_t truncated;
    uint64_t spilled;
    uint64_t queued;            /* subproblems left in the queue when a target width or budget stopped the run */
    int32_t  iterations;        /* waves (kernel iterations in the reference) */
    int32_t  n_nodes;           /* echo of the graph */
    int32_t  n_edges;
    int32_t  src, dst;
    int32_t  mask_words;
    uint64_t max_queue_items;   /* largest wave */
    double   max_queue_mb;      /* largest wave x bytes per queued subproblem */
    double   ms;                /* device time of the solve (CUDA events) */
    double   time_to_bound_ms;  /* device time until the target width was met (0 if no target) */
    int32_t  engine;            /* which engine ran (NR_ENGINE_*) */
    int32_t  grid_blocks;
    int32_t  block_threads;
    int32_t  item_bytes;        /* bytes per queued subproblem in HBM */
    uint64_t capacity;          /* queue capacity actually used (items) */
    uint64_t h2d_bytes;         /* host -> device bytes copied by this call */
    uint64_t d2h_bytes;         /* device -> host bytes copied by this call */
    int32_t  stop;              /* 0 queue empty, 1 target width met, 3 pop budget reached */
    int32_t  kernel;            /* warp engine: NR_KERNEL_GROUP, NR_KERNEL_LANE, NR_KERNEL_LANE2 or
                                   NR_KERNEL_BLOCK;
                                   whole-GPU engines: NR_KERNEL_LANE when one lane per subproblem
                                   ran (waves on <= 32 nodes; the bucketed queue on undirected
                                   simple graphs of <= 250 nodes); 0 otherwise */
    int32_t  reserved[2];
} nr_result;

enum { NR_ENGINE_GRID = 1, NR_ENGINE_WARP = 2 };

typedef struct nr_context nr_context;

/* Defaults: eps 0 (exact), no target, NR_ORDER_AUTO, shift 2, 256 buckets, device 0. */
void        nr_options_default(nr_options *opt);
const char *nr_status_string(int status);
int         nr_abi_version(void);

/* Parse a reference graph file ("N E [U|D]" then N lines "deg (nbr p)*").
 * Replaces graph_load (workingPad/graph.h:46-145) without its exit() paths;
 * also accepts files whose header has no type character (the test_*.txt
 * files).  Edge ids are first-seen (min,max) pairs (graph.h:77-90).
 * Arrays are malloc'd into *out; release with nr_graph_free. */
int  nr_graph_load(const char *path, nr_graph *out);
void nr_graph_free(nr_graph *g);

/* Initial mask of a graph: all UNKNOWN, p<=0 DOWN, p>=1 UP
 * (workingPad/main.cu:717-748). words must hold ceil(2E/32) entries. */
int  nr_initial_mask(const nr_graph *g, uint32_t *words, int n_words);

/* Reusable device state (queue buffers, stream, events). */
int  nr_context_create(int device, nr_context **out);
void nr_context_destroy(nr_context *ctx);

/* Solve one instance. capacity = queue capacity in subproblems per wave
 * buffer (the reference's --queue_capacity, main.cu:781-782); 0 picks the
 * reference default 1048576.  Replaces the body of main()
 * (workingPad/main.cu:800-1056): graph_to_device, queue_pair_init, the wave
 * loop over factoring_kernel, and the stats readback. opt may be NULL. */
int  nr_reliability(const nr_graph *g, int src, int dst, uint64_t capacity,
                    const nr_options *opt, nr_result *res);
int  nr_reliability_ctx(nr_context *ctx, const nr_graph *g, int src, int dst, uint64_t capacity,
                        const nr_options *opt, nr_result *res);

/* Solve many instances in one persistent launch (no reference counterpart:
 * the reference runs one graph per process). Instances that outgrow the
 * per-warp queue are finished by the whole-GPU engine. */
int  nr_reliability_batch(nr_context *ctx, int n_instances, const nr_graph *graphs,
                          const int32_t *srcs, const int32_t *dsts, uint64_t capacity,
                          const nr_options *opt, nr_result *results);

/* Asynchronous batches (no reference counterpart): nr_reliability_batch in
 * two halves, so the host builds one batch's tables while the GPU runs the
 * one before.  nr_batch_submit checks the batch, builds its tables and queues
 * the upload, the kernels and the read-back on one of the context's three batch
 * slots, and returns a ticket; nr_batch_wait(ticket) finishes that batch and
 * fills `results` (as given to the submit) exactly as nr_reliability_batch
 * would.  Slots take turns: a submit whose slot still holds an unfinished batch
 * finishes it first (a later wait on its ticket returns its status).  graphs,
 * srcs, dsts and results must stay valid and unchanged until the wait returns.
 * `after_stream` (a cudaStream_t, or NULL): the batch's upload starts after the
 * work already queued on that stream.  A batch with a graph above 32 nodes
 * runs to completion inside the submit. */
int  nr_batch_submit(nr_context *ctx, int n_instances, const nr_graph *graphs, const int32_t *srcs,
                     const int32_t *dsts, uint64_t capacity, const nr_options *opt, nr_result *results,
                     void *after_stream, int64_t *ticket);
int  nr_batch_wait(nr_context *ctx, int64_t ticket);

/* One topology, many probability sets (no reference counterpart: the reference runs one graph
 * per process): instance i is `topology` with edge probabilities p_matrix[i * n_edges ..
 * (i + 1) * n_edges) (topology->edge_p is not read) and terminals srcs[i], dsts[i]; n_nodes <=
 * 32.  The inputs are one matrix, so the host builds no per-instance tables: the topology is
 * checked once, the terminals per instance, and the matrix goes to the device as it is -- a
 * plain DMA when the caller allocated it pinned (cudaHostAlloc, or a pinned torch tensor) --
 * where a scan rejects NaN probabilities (NR_ERR_INVALID from the wait).  Results, tickets and
 * slots as nr_batch_submit / nr_batch_wait; p_matrix must stay valid and unchanged until the
 * wait returns. */
int  nr_batch_submit_matrix(nr_context *ctx, const nr_graph *topology, int n_instances, const double *p_matrix,
                            const int32_t *srcs, const int32_t *dsts, uint64_t capacity, const nr_options *opt,
                            nr_result *results, void *after_stream, int64_t *ticket);
int  nr_reliability_batch_matrix(nr_context *ctx, const nr_graph *topology, int n_instances,
                                 const double *p_matrix, const int32_t *srcs, const int32_t *dsts,
                                 uint64_t capacity, const nr_options *opt, nr_result *results);

/* K-terminal reliability (the reference stubs a target set, parallel/Rel_16M.cu:43): the
 * probability that every node of terminals[0..n_terminals) is connected to terminals[0].  The
 * same disjoint decomposition runs over the BFS tree that joins every terminal to terminals[0]
 * (the union of their parent paths), its UNKNOWN edges in BFS order (by depth, then node
 * index); with two terminals it is the two-terminal run exactly.  Runs on the whole-GPU
 * engines for any n <= 16384 (breadth-first waves, or the bucketed max-mass queue for
 * NR_ORDER_MAXMASS and target widths); path branching only. */
int  nr_reliability_kterminal(nr_context *ctx, const nr_graph *graph, const int32_t *terminals, int n_terminals,
                              uint64_t capacity, const nr_options *opt, nr_result *result);

/* Checkpoint / resume (no reference counterpart) of a bucketed whole-GPU run (graphs above 32
 * nodes, bucket_shift >= 0): after an nr_reliability_ctx call on the context that ran one (and
 * before another whole-GPU run on it), nr_checkpoint_save writes the live queue records, the
 * exact sums and the counts to a file.  nr_checkpoint_resume reloads them for the same graph,
 * terminals, bucket resolution, eps and branching (checked against a fingerprint in the file)
 * and continues the run with the given options -- typically a larger max_nodes or a target
 * width -- as if it had never stopped: counts, sums and waves include the work before the
 * checkpoint.  Host memory for the live records is needed on both sides. */
int  nr_checkpoint_save(nr_context *ctx, const char *path);
int  nr_checkpoint_resume(nr_context *ctx, const char *path, const nr_graph *graph, int src, int dst,
                          uint64_t capacity, const nr_options *opt, nr_result *result);

/* Autotuner for batches (no reference counterpart).  Times the warp engine on
 * up to 4096 instances of the batch for each candidate setting -- bucket
 * resolution (bucket_shift -1..2, where -1 is one bucket: breadth-first waves), pages per warp (64, 512
 * or 4096, how much of the queue a warp holds; never above capacity) and warps per block (2, 4, 8) -- and
 * writes the best into *best (based on *opt), with its device time in *best_ms:
 * the fewest instances whose queue spilled, then the shortest time (best of three runs, and
 * three more for the three leaders).  The bucket resolution is searched only for opt->order ==
 * NR_ORDER_AUTO with a target width: NR_ORDER_WAVES holds one bucket and
 * NR_ORDER_MAXMASS / NR_ORDER_LEARNED hold opt's bucket_shift and n_buckets.  Every candidate returns a valid result; the choice changes time
 * and, for truncated runs, where the stop falls. */
int  nr_autotune(nr_context *ctx, int n_instances, const nr_graph *graphs, const int32_t *srcs,
                 const int32_t *dsts, uint64_t capacity, const nr_options *opt, nr_options *best,
                 double *best_ms);

/* ---- learned scorer (no reference counterpart) ------------------------------
 * An MLP 16 -> 128 -> 128 -> 128 -> 1 (ReLU, sigmoid) estimating a
 * subproblem's residual reliability from mask features.  NR_ORDER_LEARNED
 * queues a child in the bucket of (mass x estimate) instead of mass; masses,
 * R and ESP never depend on it.  Parameters are nr_mlp_param_count() FP32
 * values: W1[128][16] b1[128] W2[128][128] b2[128] W3[128][128] b3[128]
 * w4[128] b4. */
int  nr_mlp_param_count(void);
int  nr_mlp_init(float *params, uint64_t seed);               /* He-uniform, seeded */
/* One forward + backward pass over (X[n][16], y[n]) on the GPU: mean binary
 * cross-entropy in *loss and the gradient (same layout as params) in grads. */
int  nr_mlp_grad(int device, const float *params, const float *X, const float *y, int n, float *loss, float *grads);
/* Adam on the GPU (FP32); params in: initial values, out: trained values. */
int  nr_mlp_train(int device, float *params, const float *X, const float *y, int n, int epochs, int batch,
                  float lr, float weight_decay, uint64_t seed, float *loss_per_epoch);
/* Batched inference on tensor cores (BF16 weights, FP32 accumulation). */
int  nr_mlp_infer(int device, const float *params, const float *X, int n, float *y);
/* Install parameters on a context for NR_ORDER_LEARNED. */
int  nr_context_set_model(nr_context *ctx, const float *params);
/* Run a batch like nr_reliability_batch and record every child the warp
 * engine queues (16 features, 32 mask words, mass, instance index), up to
 * max_items; training data for the scorer. */
int  nr_collect_children(nr_context *ctx, int n_instances, const nr_graph *graphs, const int32_t *srcs,
                         const int32_t *dsts, uint64_t capacity, const nr_options *opt, uint64_t max_items,
                         float *feat, uint32_t *masks, double *mass, int32_t *inst, uint64_t *count,
                         nr_result *results);

/* Solve one instance without allocating device memory (no counterpart in the
 * reference, which allocates its queues with cudaMalloc on every run).
 * For callers that cannot call cudaMalloc -- an application whose device
 * memory belongs to its own allocator or pool, or a plugin that may not grow
 * the process's device footprint -- the queue, graph tables and output live
 * in one static device array of 4 MiB per GPU, held until the process exits.
 * Limits: n_nodes <= 32 and graph tables that fit the array; larger inputs
 * return NR_ERR_UNSUPPORTED.  The queue gets the rest of the array; when it
 * is full, child mass is spilled into ESP (a valid bracket, as in the
 * reference on queue overflow).  The first call on a device looks up the
 * array's address (cudaGetSymbolAddress) and should come before any stream
 * capture.  Calls share the array: they are serialised by a lock and each
 * waits for its kernel, so anything else overlapping on the GPU that touched
 * the array would race.  Runs on cudaStreamPerThread; res->ms is in-kernel
 * device time.  capacity is not taken: the array sets it.  One warp does the
 * solve, so every run has a pop budget: opt->max_nodes, or 2^24 pops when it
 * is 0; a run that reaches it returns NR_OK with res->stop = 3 and a valid
 * bracket.  NaN probabilities return NR_ERR_INVALID.  The calling thread's
 * current device is the same after the call as before it. */
int  nr_reliability_noalloc(const nr_graph *g, int src, int dst, const nr_options *opt, nr_result *res);

/* The reference's result block (workingPad/main.cu:1037-1056) as text.
 * Returns the number of characters written (snprintf semantics). */
int  nr_format_result(const nr_result *res, char *buf, size_t len);

#ifdef __cplusplus
}
#endif
#endif /* NR_H */
