// nr_host.h -- host-side internals shared by the C ABI's translation units: the context,
// the warp engine's batch slots and run settings, status helpers, and the graph-table and
// validation helpers both the single-instance engines (nr_api.cu) and the batch runtime
// (nr_batch.cu) use.  Not part of the ABI.
#pragma once

#include <sched.h>

#include <algorithm>
#include <atomic>
#include <chrono>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <condition_variable>
#include <cstring>
#include <functional>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <vector>

#include "nr_internal.h"
#include "nr_pool.h"
#include "nr_device.cuh"
#include "nr_warp.cuh"
#include "nr_lane2.cuh"
#include "nr_grid_lane.cuh"
#include "nr_block64.cuh"
#include "nr_wide.cuh"
#include "nr_mlp.cuh"

const void *nr_grid_kernel_ptr_g8(int w4);
const void *nr_grid_fork_kernel_ptr_g8(int w4);
const void *nr_grid_fork_kernel_ptr_g16(int w4);
const void *nr_grid_fork_kernel_ptr_g32(int w4);
const void *nr_grid_kernel_ptr_g16(int w4);
const void *nr_grid_kernel_ptr_g32(int w4);
const void *nr_grid_wide_kernel_ptr(int w4);
const void *nr_bucket_wide_kernel_ptr(int w4);
const void *nr_warp_kernel_ptr_g8(int w4);
const void *nr_warp_kernel_ptr_g16(int w4);
const void *nr_warp_kernel_ptr_g32(int w4);
const void *nr_warp_learn_kernel_ptr_g8(int w4);
const void *nr_warp_fork_kernel_ptr_g8(int w4);
const void *nr_warp_fork_kernel_ptr_g16(int w4);
const void *nr_warp_fork_kernel_ptr_g32(int w4);
const void *nr_warp_learn_kernel_ptr_g16(int w4);
const void *nr_warp_learn_kernel_ptr_g32(int w4);
const void *nr_lane_kernel_ptr(int w4);
const void *nr_grid_lane_kernel_ptr(int w4, int row_bits = 16);
const void *nr_grid_wide_multi_kernel_ptr(int w4);
const void *nr_bucket_wide_learn_kernel_ptr(int w4);
const void *nr_bucket_wide_lanes_kernel_ptr(int w4);
int run_grid_wide_multi(nr_context *c, const std::vector<int> &idx, const nr_graph *gs, const int32_t *srcs,
                        const int32_t *dsts, uint64_t cap, const nr_options *o, nr_result *res);
const void *nr_lane2_kernel_ptr(int w4, int slots, int row_bits = 16);
const void *nr_block_lane_kernel_ptr(int w4, int row_bits);
const void *nr_block64_kernel_ptr(int w4);
int nr_mlp_upload(const float *params, void **storage, NrMlpDev *out, cudaStream_t s);

#define NR_CUDA_TRY(call)                                                     \
    do {                                                                      \
        cudaError_t _e = (call);                                              \
        if (_e != cudaSuccess) {                                              \
            nr_last_cuda_error(_e, __FILE__, __LINE__, #call);                \
            return NR_ERR_CUDA;                                               \
        }                                                                     \
    } while (0)

extern thread_local char g_err[256];
extern thread_local char g_internal[128];      // which device-side check failed, when one says
// keep the failing call and its line for nr_status_string
void nr_last_cuda_error(cudaError_t e, const char *file, int line, const char *what);

inline const void *grid_kernel(int G, int w4, bool fork = false)
{
    switch (G) {
    case 8: return fork ? nr_grid_fork_kernel_ptr_g8(w4) : nr_grid_kernel_ptr_g8(w4);
    case 16: return fork ? nr_grid_fork_kernel_ptr_g16(w4) : nr_grid_kernel_ptr_g16(w4);
    case 32: return fork ? nr_grid_fork_kernel_ptr_g32(w4) : nr_grid_kernel_ptr_g32(w4);
    default: return nullptr;
    }
}

inline const void *warp_kernel(int G, int w4, bool learn = false, bool fork = false)
{
    switch (G) {
    case 8: return learn ? nr_warp_learn_kernel_ptr_g8(w4) : fork ? nr_warp_fork_kernel_ptr_g8(w4)
                                                                 : nr_warp_kernel_ptr_g8(w4);
    case 16: return learn ? nr_warp_learn_kernel_ptr_g16(w4) : fork ? nr_warp_fork_kernel_ptr_g16(w4)
                                                                   : nr_warp_kernel_ptr_g16(w4);
    case 32: return learn ? nr_warp_learn_kernel_ptr_g32(w4) : fork ? nr_warp_fork_kernel_ptr_g32(w4)
                                                                   : nr_warp_kernel_ptr_g32(w4);
    default: return nullptr;
    }
}

inline int group_width(int n)
{
    if (n <= 8) return 8;
    if (n <= 16) return 16;
    return 32;
}

inline size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

// NR_PROFILE=1 in the environment: host phase timings of batch calls on stderr
struct PhaseClock {
    bool on;
    std::chrono::steady_clock::time_point t0, last;
    char buf[512];
    int len = 0;
    PhaseClock() : on(getenv("NR_PROFILE") != nullptr)
    {
        t0 = last = std::chrono::steady_clock::now();
        buf[0] = 0;
    }
    void mark(const char *name)
    {
        if (!on) return;
        const auto t = std::chrono::steady_clock::now();
        len += snprintf(buf + len, sizeof(buf) - len, " %s=%.1fus", name,
                        std::chrono::duration<double, std::micro>(t - last).count());
        last = t;
    }
    ~PhaseClock()
    {
        if (on) fprintf(stderr, "[nr profile]%s total=%.1fus\n", buf,
                        std::chrono::duration<double, std::micro>(std::chrono::steady_clock::now() - t0).count());
    }
};




// One host block of a batch call (a contiguous instance range): table bytes,
// instances per class, and where its tables and descriptors go.
#define NR_HOST_BLOCKS 64
// warp-engine kernel classes: lane-group width (8, 16, 32) x mask blocks, then the
// one-lane-per-subproblem kernel x mask blocks
#define NR_LANE_CLS0 (3 * NR_MAX_W4)
// then the two-slot lane kernel with 32-bit rows (17..32 nodes) x mask blocks
#define NR_LANE32_MAX_W4 8      // a simple graph on <= 32 nodes has <= 496 edges: 31 mask words
#define NR_LANE32_CLS0 (NR_LANE_CLS0 + NR_LANE_MAX_W4)
#define NR_NCLS (NR_LANE32_CLS0 + NR_LANE32_MAX_W4)
// the two-slot lane kernel hands an instance to the block kernel once its next wave holds more
// than this many pages (256 subproblems: one step of the block's 256 lanes).  On the uneven
// batch's 3,959 graphs of <= 32 nodes: 8 pages 13.0 ms, 16 13.6-14.0, 32 15.7, 64 17.6-18.6, 128
// 22.9-24.7, never 59-72 ms; 4,096 K15 or 1,024 K25 instances never reach it (widest waves 32).
#define NR_HANDOVER_PAGES 8
struct NrHostBlock {
    size_t bytes;               // tables of the block's instances (16-byte multiples)
    long long last_owner_rel;   // offset in the block of its last structural part, -1 if none
    size_t base;                // offset of the block's tables in the staging buffer
    long long struct_in;        // struct_off of the last structural part before the block
    int last_rows;              // rows mode of the block's last structural part, -1 if none
    int rows_in;                // rows mode of the last structural part before the block
    int cnt[NR_NCLS];           // instances per class
    int cbase[NR_NCLS];         // instances of each class in earlier blocks
};

// Host-side per-instance tables of a batch call, kept by the context so their
// memory is reused from call to call.
struct NrBatchScratch {
    std::vector<NrSmallGraph> desc;
    std::vector<int> cls;
    std::vector<unsigned char> same_prev;
    std::vector<size_t> inst_b, struct_b;
    std::vector<NrHostBlock> blk;
};

struct WarpDump;
struct WarpRunCfg {
    int wave_mode, shift, n_buckets, pages, escalate, warps_per_block;
    int fork = 0;
    int learned = 0;
    int lane = 1;                 // one lane per subproblem where it applies
    int lane2 = 1;                // ... with several instances per warp in breadth-first waves
    int lane_slots = 2;           // instances per warp then
    long long step_cap = 0;       // lane kernels' step bound (0: the kernels' own; tests set 1)
    int border = NR_BORDER_SRC;   // branch order of the paths' UNKNOWN edges
    int handover_pages = 0;       // two-slot lane kernel: hand-over to the block kernel (0 = never)
    const WarpDump *dump = nullptr;
    double eps, target;
    unsigned long long max_nodes;
};

// A warp-engine batch in flight: its stream, staging, device tables and page
// slabs.  A context has NR_SLOTS, used in turn by nr_batch_submit, so one batch's
// tables are built on the host while the batch before runs.  (Splitting one
// batch over both slots measured slower on 4096 K15 instances: the host passes
// are dominated by fixed costs and two concurrent launches lengthen the span.)
#define NR_SLOTS 3
#define NR_HV_STREAMS 4
struct NrSlot {
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;   // around the part's kernels
    void *hbuf = nullptr;       // pinned host staging for the uploads and results
    size_t hbuf_bytes = 0;
    void *wbuf = nullptr;       // device: counters, tables, descriptors, ids, outputs
    size_t wbuf_bytes = 0;
    void *wslab = nullptr;      // device: per-warp page slabs
    size_t wslab_bytes = 0;
    NrBatchScratch scratch;     // per-instance host tables (reused from call to call)
    void *hv_host = nullptr;    // instances handed to the block kernel: pinned staging ...
    size_t hv_host_bytes = 0;
    void *hv_dev = nullptr;     // ... and device copies of their descriptors, ids and outputs
    size_t hv_dev_bytes = 0;
    cudaStream_t hv_side[NR_HV_STREAMS] = {};   // their launches, one class a stream, side by side
    cudaEvent_t hv_fork = nullptr, hv_join[NR_HV_STREAMS] = {};
    // the part queued by warp_submit, for warp_finish
    int n = 0;
    const nr_graph *gs = nullptr;
    const int32_t *srcs = nullptr, *dsts = nullptr;
    nr_result *res = nullptr;
    WarpRunCfg cfgp{};
    size_t off_out = 0;
    int first_grid = 0, block = 0;
    int nps[NR_NCLS] = {0};     // pages a warp held, per kernel class
    bool matrix = false;        // one topology, the caller's probability matrix (gs[0] for every instance)
    const double *pmat = nullptr;
    size_t off_flag = 0;        // matrix batches: the NaN flag the device scan sets
    // asynchronous batches: the ticket queued here and what its wait needs
    int64_t ticket = 0;
    bool pending = false;
    uint64_t capacity = 0;
    nr_options opt{};
};

// What a checkpoint of the last bucketed whole-GPU run needs (its queue stays in the
// context's arena until another whole-GPU run reuses it).
struct NrCkptState {
    bool valid = false;
    uint64_t fp = 0;                 // graph, terminals and options
    int n = 0, E = 0, src = 0, dst = 0, W4 = 0;
    NrFix R{}, et{}, es{}, net{};
    unsigned long long nodes = 0, leaves = 0, dead = 0, trunc = 0, spilled = 0, max_wave = 0;
    long long waves = 0;
    unsigned long long cap = 0;      // arena slots
    size_t mask_bytes = 0, mass_bytes = 0;
    size_t off_top = 0;              // arena top in the control buffer
};

// A checkpoint to resume from: the live records and the sums and counts so far.
struct NrResumeIn {
    std::vector<unsigned char> masks;  // [live][W4 * 16]
    std::vector<double> mass;          // [live]
    NrFix R{}, et{}, es{}, net{};
    unsigned long long nodes = 0, leaves = 0, dead = 0, trunc = 0, spilled = 0, max_wave = 0;
    long long waves = 0;
};

struct nr_context {
    int device = 0;
    int sms = 0;
    cudaStream_t stream = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    void *qbuf = nullptr;       // ping-pong wave buffers
    size_t qbytes = 0;
    void *sbuf = nullptr;       // blob, counters, barrier, status, partials
    size_t sbytes = 0;
    NrSlot slot[NR_SLOTS];      // warp engine: one per part of a batch in flight
    std::map<std::pair<const void *, size_t>, int> occupancy;   // (kernel, smem) -> blocks per SM
    std::unique_ptr<NrPool> pool;   // host worker threads, created by the first large batch
    int64_t next_ticket = 1;        // asynchronous batches
    std::map<int64_t, int> done_rc; // status of batches finished before their wait
    cudaEvent_t ev_after = nullptr; // orders a batch after a caller's stream
    NrCkptState ckpt;               // the last bucketed whole-GPU run
    int smem_optin = 0;             // largest dynamic shared memory a block may opt in to
    void *model = nullptr;          // learned scorer: FP32 parameters and their BF16 copy
    NrMlpDev mlp{};
    bool has_model = false;
    std::mutex mu;

    // run fn(i) for i in [0, n): serially when n < 2 * min_per_thread, else on the
    // worker pool with at most one thread per min_per_thread indices
    void parallel_for(int n, int min_per_thread, const std::function<void(int)> &fn)
    {
        if (n < 2 * min_per_thread) {
            for (int i = 0; i < n; ++i) fn(i);
            return;
        }
        if (!pool) {
            // the CPUs this process may run on (a container can get fewer than the machine has)
            cpu_set_t set;
            int hw = 0;
            if (sched_getaffinity(0, sizeof(set), &set) == 0) hw = CPU_COUNT(&set);
            if (hw <= 0) hw = (int)std::thread::hardware_concurrency();
            hw = std::max(1, std::min(hw, NR_POOL_MAX));
            pool.reset(new NrPool(hw - 1));
        }
        const int threads = std::min(pool->size(), (n + min_per_thread - 1) / min_per_thread);
        // about four grabs per thread: enough to even out uneven items, few enough that the
        // shared counter is not the cost
        pool->run(n, threads - 1, std::max(1, std::min(256, n / (4 * threads))), fn);
    }
};

struct WarpDump {
    float *feat;                     // device buffers (nullptr: no dump)
    uint32_t *mask;
    double *mass;
    int *inst;
    unsigned long long *count;
    unsigned long long cap;
    int stride;
};

// nr_api.cu
int ensure(void **buf, size_t *have, size_t need);
int validate_shape(const nr_graph *g, int src, int dst);
int validate_probabilities(const nr_graph *g);
int validate_structure(const nr_graph *g);
bool same_structure_arrays(const nr_graph *a, const nr_graph *b);
int validate(const nr_graph *g, int src, int dst);
int rows_mode_of(const nr_graph *g);
size_t small_inst_layout(const nr_graph *g, int src, int dst, NrSmallGraph *sg);
size_t small_struct_layout(const nr_graph *g, NrSmallGraph *sg, size_t at);
bool small_fill_inst(const nr_graph *g, const NrSmallGraph *sg, unsigned char *b);
void small_fill_struct(const nr_graph *g, const NrSmallGraph *sg, unsigned char *b);
bool same_topology(const nr_graph *a, const nr_graph *b);
int smem_optin(nr_context *c);
int run_grid_small(nr_context *c, const nr_graph *g, int src, int dst, uint64_t cap, const nr_options *o,
                   nr_result *r);
int run_wide(nr_context *c, const nr_graph *g, int src, int dst, uint64_t capacity, const nr_options *o,
             nr_result *r, const int32_t *terms = nullptr, int nt = 0);

// nr_batch.cu
WarpRunCfg warp_cfg(const nr_options *o, uint64_t capacity, bool exhaustive);
int run_warp_batch(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                   const WarpRunCfg &cfg, nr_result *res, std::vector<int> *handover, PhaseClock *clock = nullptr);
int branch_order_ok(const nr_context *c, const nr_options &o);
void drain(nr_context *c);
