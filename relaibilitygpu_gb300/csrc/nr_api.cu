// nr_api.cu -- host side of the C ABI declared in include/nr.h.
//
// Replaces the reference driver (workingPad/main.cu:795-1072) and its graph
// loader (workingPad/graph.h:46-178) with calls that return status codes.

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
const void *nr_lane2_kernel_ptr(int w4, int slots);
int nr_mlp_upload(const float *params, void **storage, NrMlpDev *out, cudaStream_t s);

namespace {

#define NR_CUDA_TRY(call)                                                     \
    do {                                                                      \
        cudaError_t _e = (call);                                              \
        if (_e != cudaSuccess) {                                              \
            nr_last_cuda_error(_e, __LINE__, #call);                          \
            return NR_ERR_CUDA;                                               \
        }                                                                     \
    } while (0)

thread_local char g_err[256];
thread_local char g_internal[128];      // which device-side check failed, when one says

// keep the failing call and its line for nr_status_string
void nr_last_cuda_error(cudaError_t e, int line, const char *what)
{
    snprintf(g_err, sizeof(g_err), "%s (nr_api.cu:%d %.120s)", cudaGetErrorString(e), line, what);
}

const void *grid_kernel(int G, int w4, bool fork = false)
{
    switch (G) {
    case 8: return fork ? nr_grid_fork_kernel_ptr_g8(w4) : nr_grid_kernel_ptr_g8(w4);
    case 16: return fork ? nr_grid_fork_kernel_ptr_g16(w4) : nr_grid_kernel_ptr_g16(w4);
    case 32: return fork ? nr_grid_fork_kernel_ptr_g32(w4) : nr_grid_kernel_ptr_g32(w4);
    default: return nullptr;
    }
}

const void *warp_kernel(int G, int w4, bool learn = false, bool fork = false)
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

int group_width(int n)
{
    if (n <= 8) return 8;
    if (n <= 16) return 16;
    return 32;
}

size_t align16(size_t x) { return (x + 15) & ~size_t(15); }

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

}  // namespace

// Dynamic shared-memory limit of a kernel on a device: the attribute is
// per-function state, so every setter in the library goes through here and
// the attribute is set only when it differs from the value last set.
cudaError_t nr_smem_limit(int device, const void *kfn, size_t bytes)
{
    static std::mutex mu;
    static std::map<std::pair<int, const void *>, size_t> last;
    std::lock_guard<std::mutex> l(mu);
    auto it = last.find({device, kfn});
    if (it != last.end() && it->second == bytes) return cudaSuccess;
    const cudaError_t e = cudaFuncSetAttribute(kfn, cudaFuncAttributeMaxDynamicSharedMemorySize, (int)bytes);
    if (e == cudaSuccess) last[{device, kfn}] = bytes;
    else last.erase({device, kfn});
    return e;
}

// Correctly rounded (to nearest, ties to even) value of a 192-bit fixed-point sum.
double nr_fix_to_double_host(const NrFix &a)
{
    const unsigned long long w[3] = {a.w0, a.w1, a.w2};
    int i = 2;
    while (i >= 0 && w[i] == 0ull) --i;
    if (i < 0) return 0.0;
    const int t = 64 * i + 63 - __builtin_clzll(w[i]);   // top set bit
    unsigned long long x;
    bool sticky = false;
    if (t >= 63) {
        const int lo = t - 63, k = lo >> 6, b = lo & 63;
        x = w[k] >> b;
        if (b && k + 1 < 3) x |= w[k + 1] << (64 - b);
        if (b) sticky = (w[k] & ((1ull << b) - 1ull)) != 0ull;
        for (int j = 0; j < k; ++j) sticky = sticky || w[j] != 0ull;
    } else {
        x = w[0] << (63 - t);
    }
    unsigned long long mant = x >> 11;
    const unsigned long long rem = x & 0x7ffull;
    int top = t;
    if (rem > 0x400ull || (rem == 0x400ull && (sticky || (mant & 1ull)))) {
        ++mant;
        if (mant >> 53) { mant >>= 1; ++top; }
    }
    // mant in [2^52, 2^53): the value is mant * 2^(top - 52 - NR_FIX_FRAC), a normal double
    // (top <= 191 and NR_FIX_FRAC = 190 keep the exponent well inside the normal range)
    const unsigned long long bits = ((unsigned long long)(top - NR_FIX_FRAC + 1023) << 52) |
                                    (mant & 0xfffffffffffffull);
    double d;
    memcpy(&d, &bits, sizeof d);
    return d;
}

NrFix nr_fix_from_double_host(double m) { return nr_fix_of(m); }
void nr_fix_add_host(NrFix &a, const NrFix &b) { nr_fix_add(a, b); }



// One host block of a batch call (a contiguous instance range): table bytes,
// instances per class, and where its tables and descriptors go.
#define NR_HOST_BLOCKS 64
// warp-engine kernel classes: lane-group width (8, 16, 32) x mask blocks, then the
// one-lane-per-subproblem kernel x mask blocks
#define NR_LANE_CLS0 (3 * NR_MAX_W4)
#define NR_NCLS (NR_LANE_CLS0 + NR_LANE_MAX_W4)
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
    const WarpDump *dump = nullptr;
    double eps, target;
    unsigned long long max_nodes;
};

// A warp-engine batch in flight: its stream, staging, device tables and page
// slabs.  A context has two, used in turn by nr_batch_submit, so one batch's
// tables are built on the host while the batch before runs.  (Splitting one
// batch over both slots measured slower on 4096 K15 instances: the host passes
// are dominated by fixed costs and two concurrent launches lengthen the span.)
#define NR_SLOTS 2
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
    // the part queued by warp_submit, for warp_finish
    int n = 0;
    const nr_graph *gs = nullptr;
    const int32_t *srcs = nullptr, *dsts = nullptr;
    nr_result *res = nullptr;
    WarpRunCfg cfgp{};
    size_t off_out = 0;
    int first_grid = 0, block = 0;
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

// Sets *flag when any of the n doubles is a NaN (integer test of the bit pattern).
__global__ void nr_nan_scan_kernel(const unsigned long long *p, size_t n, int *flag)
{
    int hit = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        hit |= (p[i] & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
    if (__syncthreads_or(hit) && threadIdx.x == 0) *flag = 1;
}

static cudaError_t nr_launch_nan_scan(const double *p, size_t n, int *flag, cudaStream_t s)
{
    if (!n) return cudaSuccess;
    const int block = 256;
    const int grid = (int)std::min<size_t>((n + block - 1) / block, 1024);
    nr_nan_scan_kernel<<<grid, block, 0, s>>>(reinterpret_cast<const unsigned long long *>(p), n, flag);
    return cudaGetLastError();
}

static int ensure(void **buf, size_t *have, size_t need)
{
    if (*have >= need && *buf) return NR_OK;
    if (*buf) cudaFree(*buf);
    *buf = nullptr;
    *have = 0;
    cudaError_t e = cudaMalloc(buf, need);
    if (e != cudaSuccess) {
        cudaGetLastError();
        *buf = nullptr;
        return (e == cudaErrorMemoryAllocation) ? NR_ERR_NOMEM : NR_ERR_CUDA;
    }
    *have = need;
    return NR_OK;
}

// ---------------------------------------------------------------------------
// validation and graph tables
// ---------------------------------------------------------------------------
// Checks of one instance that read no array: sizes, pointers, terminals.
static int validate_shape(const nr_graph *g, int src, int dst)
{
    if (!g || g->n_nodes <= 0 || g->n_edges < 0 || g->n_arcs < 0 || !g->row_ptr) return NR_ERR_INVALID;
    if (g->n_arcs > 0 && (!g->col_idx || !g->edge_id)) return NR_ERR_INVALID;
    if (g->n_edges > 0 && !g->edge_p) return NR_ERR_INVALID;
    if (src < 0 || dst < 0 || src >= g->n_nodes || dst >= g->n_nodes) return NR_ERR_INVALID;
    return NR_OK;
}

static int validate_probabilities(const nr_graph *g)
{
    for (int e = 0; e < g->n_edges; ++e)
        if (std::isnan(g->edge_p[e])) return NR_ERR_INVALID;
    return NR_OK;
}

// The CSR arrays: row offsets, heads and edge ids in range.
static int validate_structure(const nr_graph *g)
{
    if (g->row_ptr[0] != 0 || g->row_ptr[g->n_nodes] != g->n_arcs) return NR_ERR_INVALID;
    for (int u = 0; u < g->n_nodes; ++u)
        if (g->row_ptr[u + 1] < g->row_ptr[u]) return NR_ERR_INVALID;
    for (int j = 0; j < g->n_arcs; ++j) {
        if (g->col_idx[j] < 0 || g->col_idx[j] >= g->n_nodes) return NR_ERR_INVALID;
        if (g->edge_id[j] < 0 || g->edge_id[j] >= g->n_edges) return NR_ERR_INVALID;
    }
    return NR_OK;
}

// Same sizes and the same CSR arrays (pointers) as another graph.
static bool same_structure_arrays(const nr_graph *a, const nr_graph *b)
{
    return a->n_nodes == b->n_nodes && a->n_arcs == b->n_arcs && a->n_edges == b->n_edges &&
           a->row_ptr == b->row_ptr && a->col_idx == b->col_idx && a->edge_id == b->edge_id;
}

static int validate(const nr_graph *g, int src, int dst)
{
    int rc = validate_shape(g, src, dst);
    if (!rc) rc = validate_probabilities(g);
    if (!rc) rc = validate_structure(g);
    return rc;
}

static int group_width_of(int n) { return group_width(n); }

// Whether the warp engine can carry not-down in-neighbour rows in its queue
// records (a child's rows are its parent's less the arcs of its down edge):
// 1 for an undirected simple graph (every edge id on exactly two arcs, u -> v and
// v -> u), 2 for a directed simple graph (one arc per edge id), 0 otherwise
// (self-loops, or one ordered pair with two edge ids); 0 makes it rebuild rows.
static int rows_mode_of(const nr_graph *g)
{
    const int n = g->n_nodes, E = g->n_edges;
    if (n > NR_SMALL_MAX_N) return 0;
    static thread_local int pid[NR_SMALL_MAX_N][NR_SMALL_MAX_N];
    for (int u = 0; u < n; ++u)
        for (int v = 0; v < n; ++v) pid[u][v] = -1;
    std::vector<int> cnt(std::max(E, 1), 0);
    for (int u = 0; u < n; ++u)
        for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; ++j) {
            const int v = g->col_idx[j], e = g->edge_id[j];
            if (v == u) return 0;
            if (pid[u][v] != -1 && pid[u][v] != e) return 0;
            if (pid[u][v] == e) return 0;                 // the same arc twice
            pid[u][v] = e;
            cnt[e]++;
        }
    bool all1 = true, all2 = true;
    for (int e = 0; e < E; ++e) {
        all1 = all1 && cnt[e] == 1;
        all2 = all2 && cnt[e] == 2;
    }
    if (all1) return 2;
    if (!all2) return 0;
    for (int u = 0; u < n; ++u)
        for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; ++j)
            if (pid[g->col_idx[j]][u] != g->edge_id[j]) return 0;   // the other arc is not v -> u
    return 1;
}

// Graph tables of one instance for the small engines (layout in nr_internal.h).
// Per-instance part: the offset of p from its own base.
static size_t small_inst_layout(const nr_graph *g, int src, int dst, NrSmallGraph *sg)
{
    const int n = g->n_nodes, E = g->n_edges;
    const int W = std::max(1, (2 * E + 31) / 32);
    sg->n = n; sg->e = E; sg->w4 = (W + 3) / 4; sg->src = src; sg->dst = dst;
    sg->n_in = g->n_arcs;
    sg->rows = 0;
    sg->off_rows16 = 0;
    size_t off = 0;
    sg->off_p = (int)off; off = align16(off + sizeof(double) * std::max(E, 1));
    return off;
}

// Structural part: offsets of the edge-id table and in-arc lists from base `at`.
static size_t small_struct_layout(const nr_graph *g, NrSmallGraph *sg, size_t at)
{
    const int n = g->n_nodes, G = group_width_of(n);
    size_t off = at;
    sg->off_eid = (int)off; off = align16(off + sizeof(uint16_t) * G * G);
    sg->off_start = (int)off; off = align16(off + sizeof(int) * (n + 1));
    sg->off_list = (int)off; off = align16(off + sizeof(uint32_t) * std::max(g->n_arcs, 1));
    sg->off_rows16 = (int)off; off = align16(off + sizeof(uint32_t) * 8);
    return off - at;
}

// Copies p; false if one of them is NaN.
static bool small_fill_inst(const nr_graph *g, const NrSmallGraph *sg, unsigned char *b)
{
    const int E = g->n_edges;
    double *p = reinterpret_cast<double *>(b + sg->off_p);
    memcpy(p, g->edge_p, sizeof(double) * E);
    int nan = 0;
    for (int e = 0; e < E; ++e) nan |= p[e] != p[e];     // no early exit: the loop vectorizes
    return nan == 0;
}

static void small_fill_struct(const nr_graph *g, const NrSmallGraph *sg, unsigned char *b)
{
    const int n = g->n_nodes, G = group_width_of(n);
    uint16_t *eid = reinterpret_cast<uint16_t *>(b + sg->off_eid);
    int *start = reinterpret_cast<int *>(b + sg->off_start);
    uint32_t *list = reinterpret_cast<uint32_t *>(b + sg->off_list);
    for (int i = 0; i < G * G; ++i) eid[i] = 0xffff;
    // in-arcs grouped by head node; arc (u -> v) for every CSR entry of u
    int cnt[NR_SMALL_MAX_N + 1] = {0};
    for (int u = 0; u < n; ++u)
        for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; ++j) cnt[g->col_idx[j] + 1]++;
    for (int v = 0; v < n; ++v) cnt[v + 1] += cnt[v];
    for (int v = 0; v <= n; ++v) start[v] = cnt[v];
    int fill[NR_SMALL_MAX_N] = {0};
    for (int u = 0; u < n; ++u)
        for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; ++j) {
            const int v = g->col_idx[j], e = g->edge_id[j];
            list[start[v] + fill[v]++] = ((uint32_t)e << 8) | (uint32_t)u;
            if (eid[u * G + v] == 0xffff) eid[u * G + v] = (uint16_t)e;   // first arc u->v in CSR order
        }
    // n <= 16: the rows of the lane kernel's root when no edge is certainly down
    uint32_t *rows16 = reinterpret_cast<uint32_t *>(b + sg->off_rows16);
    for (int k = 0; k < 8; ++k) rows16[k] = 0u;
    if (n <= 16)
        for (int u = 0; u < n; ++u)
            for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; ++j) {
                const int v = g->col_idx[j];
                rows16[v >> 1] |= 1u << (u + ((v & 1) << 4));
            }
}

// Both parts in one blob (whole-GPU engine): struct_off == blob_off.
static size_t small_layout(const nr_graph *g, int src, int dst, NrSmallGraph *sg)
{
    const size_t a = small_inst_layout(g, src, dst, sg);
    const size_t b = small_struct_layout(g, sg, a);
    sg->blob_bytes = (int)(a + b);
    sg->blob_off = 0;
    sg->struct_off = 0;
    return a + b;
}

static void small_fill(const nr_graph *g, const NrSmallGraph *sg, unsigned char *b)
{
    small_fill_inst(g, sg, b);
    small_fill_struct(g, sg, b);
}

// Same topology (CSR and edge ids) as another graph?
static bool same_topology(const nr_graph *a, const nr_graph *b)
{
    if (a->n_nodes != b->n_nodes || a->n_arcs != b->n_arcs || a->n_edges != b->n_edges) return false;
    const size_t na = (size_t)a->n_arcs;
    return (a->row_ptr == b->row_ptr || !memcmp(a->row_ptr, b->row_ptr, sizeof(int32_t) * (a->n_nodes + 1))) &&
           (a->col_idx == b->col_idx || !memcmp(a->col_idx, b->col_idx, sizeof(int32_t) * na)) &&
           (a->edge_id == b->edge_id || !memcmp(a->edge_id, b->edge_id, sizeof(int32_t) * na));
}

static void build_small_blob(const nr_graph *g, int src, int dst, NrSmallGraph *sg, std::vector<unsigned char> *blob)
{
    const size_t bytes = small_layout(g, src, dst, sg);
    blob->assign(bytes, 0);
    small_fill(g, sg, blob->data());
}

extern "C" int nr_initial_mask(const nr_graph *g, uint32_t *words, int n_words)
{
    if (!g || !words || g->n_edges < 0) return NR_ERR_INVALID;
    const int W = std::max(1, (2 * g->n_edges + 31) / 32);
    if (n_words < W) return NR_ERR_INVALID;
    for (int i = 0; i < n_words; ++i) words[i] = 0;
    for (int e = 0; e < g->n_edges; ++e) {
        const double p = g->edge_p[e];
        uint32_t st = (p <= 0.0) ? NR_EDGE_DOWN : (p >= 1.0) ? NR_EDGE_UP : NR_EDGE_UNKNOWN;
        words[e >> 4] |= st << ((e & 15) * 2);
    }
    return NR_OK;
}

// ---------------------------------------------------------------------------
// public API
// ---------------------------------------------------------------------------
extern "C" void nr_options_default(nr_options *o)
{
    if (!o) return;
    memset(o, 0, sizeof(*o));
    o->order = NR_ORDER_AUTO;
    o->bucket_shift = 2;
    o->n_buckets = 256;
    o->device = 0;
    o->timeout_ms = 60000.0;
}

extern "C" int nr_abi_version(void) { return NR_ABI_VERSION; }

extern "C" const char *nr_status_string(int s)
{
    switch (s) {
    case NR_OK: return "ok";
    case NR_ERR_INVALID: return "invalid argument";
    case NR_ERR_IO: return "cannot read graph file";
    case NR_ERR_PARSE: return "malformed graph file";
    case NR_ERR_UNSUPPORTED: return "graph outside engine limits";
    case NR_ERR_CUDA: return g_err[0] ? g_err : "CUDA error";
    case NR_ERR_NOMEM: return "out of memory";
    case NR_ERR_TIMEOUT: return "device wait timed out";
    case NR_ERR_INTERNAL: return g_internal[0] ? g_internal : "internal consistency check failed";
    default: return "unknown status";
    }
}

extern "C" int nr_context_create(int device, nr_context **out)
{
    if (!out) return NR_ERR_INVALID;
    *out = nullptr;
    int ndev = 0;
    NR_CUDA_TRY(cudaGetDeviceCount(&ndev));
    if (device < 0 || device >= ndev) return NR_ERR_INVALID;
    NR_CUDA_TRY(cudaSetDevice(device));
    nr_context *c = new nr_context();
    c->device = device;
    cudaDeviceProp prop;
    cudaError_t e = cudaGetDeviceProperties(&prop, device);
    if (e == cudaSuccess) e = cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&c->ev1);
    if (e != cudaSuccess) {
        nr_last_cuda_error(e, __LINE__, "context set-up");
        nr_context_destroy(c);
        return NR_ERR_CUDA;
    }
    c->sms = prop.multiProcessorCount;
    *out = c;
    return NR_OK;
}

extern "C" void nr_context_destroy(nr_context *c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    if (c->qbuf) cudaFree(c->qbuf);
    if (c->sbuf) cudaFree(c->sbuf);
    for (NrSlot &sl : c->slot) {
        if (sl.stream) cudaStreamSynchronize(sl.stream);   // a batch submitted and never waited for
        if (sl.wslab) cudaFree(sl.wslab);
        if (sl.wbuf) cudaFree(sl.wbuf);
        if (sl.hbuf) cudaFreeHost(sl.hbuf);
        if (sl.ev0) cudaEventDestroy(sl.ev0);
        if (sl.ev1) cudaEventDestroy(sl.ev1);
        if (sl.stream) cudaStreamDestroy(sl.stream);
    }
    if (c->model) cudaFree(c->model);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->ev_after) cudaEventDestroy(c->ev_after);
    if (c->stream) cudaStreamDestroy(c->stream);
    delete c;
}

static int run_grid_small(nr_context *c, const nr_graph *g, int src, int dst, uint64_t cap,
                          const nr_options *o, nr_result *r)
{
    c->ckpt.valid = false;                 // the arena is about to be reused
    NrSmallGraph sg;
    std::vector<unsigned char> blob;
    build_small_blob(g, src, dst, &sg, &blob);
    const int G = group_width(g->n_nodes);
    const int W4 = sg.w4;
    if (W4 > NR_MAX_W4) return NR_ERR_UNSUPPORTED;
    const void *kfn = grid_kernel(G, W4, o->branching == NR_BRANCH_FORK);
    if (!kfn) return NR_ERR_UNSUPPORTED;

    const int block = NR_BLOCK_THREADS;
    const int warps = block / 32;
    const size_t smem = (size_t)sg.blob_bytes + (size_t)warps * (32 / G) * 4 * W4 * sizeof(uint32_t);
    NR_CUDA_TRY(nr_smem_limit(c->device, kfn, smem));
    int bps = 0;
    NR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kfn, block, smem));
    if (bps < 1) return NR_ERR_UNSUPPORTED;
    if (o->blocks_per_sm > 0 && o->blocks_per_sm < bps) bps = o->blocks_per_sm;
    const int grid = bps * c->sms;

    const size_t item_bytes = (size_t)W4 * 16 + sizeof(double);
    const size_t mask_bytes = align16((size_t)cap * W4 * 16);
    const size_t mass_bytes = align16((size_t)cap * sizeof(double));
    const size_t qneed = 2 * (mask_bytes + mass_bytes);
    size_t free_b = 0, total_b = 0;
    NR_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    if (qneed > c->qbytes && qneed > free_b + c->qbytes) return NR_ERR_NOMEM;
    int rc = ensure(&c->qbuf, &c->qbytes, qneed);
    if (rc) return rc;

    const int max_waves = g->n_edges + 2;
    size_t off = 0;
    const size_t off_blob = off; off = align16(off + blob.size());
    const size_t off_wc = off; off = align16(off + sizeof(unsigned long long) * (max_waves + 1));
    const size_t off_bar = off; off = align16(off + 4 * sizeof(unsigned));
    const size_t off_part = off; off = align16(off + sizeof(NrPartial) * grid);
    rc = ensure(&c->sbuf, &c->sbytes, off);
    if (rc) return rc;
    unsigned char *sb = static_cast<unsigned char *>(c->sbuf);
    unsigned char *qb = static_cast<unsigned char *>(c->qbuf);

    NrGridParams P;
    P.g = sg;
    P.blob = sb + off_blob;
    P.mask[0] = reinterpret_cast<uint4 *>(qb);
    P.mass[0] = reinterpret_cast<double *>(qb + mask_bytes);
    P.mask[1] = reinterpret_cast<uint4 *>(qb + mask_bytes + mass_bytes);
    P.mass[1] = reinterpret_cast<double *>(qb + 2 * mask_bytes + mass_bytes);
    P.capacity = cap;
    P.wave_count = reinterpret_cast<unsigned long long *>(sb + off_wc);
    P.max_waves = max_waves;
    P.bar_count = reinterpret_cast<unsigned *>(sb + off_bar);
    P.bar_gen = P.bar_count + 1;
    P.status = reinterpret_cast<int *>(P.bar_count + 2);
    P.partials = reinterpret_cast<NrPartial *>(sb + off_part);
    P.eps = o->truncation_eps > 0 ? o->truncation_eps : 0.0;
    P.timeout_ns = (long long)((o->timeout_ms > 0 ? o->timeout_ms : 60000.0) * 1e6);
    P.fork = (o->branching == NR_BRANCH_FORK);
    P.test_fault = (o->test_fault == 1);
    P.border = o->branch_order;

    // root subproblem: initial mask with mass 1 (main.cu:805-809)
    std::vector<uint32_t> root(4 * W4, 0);
    nr_initial_mask(g, root.data(), 4 * W4);
    const double one = 1.0;
    const unsigned long long one_u = 1;
    cudaStream_t s = c->stream;
    NR_CUDA_TRY(cudaMemcpyAsync(sb + off_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice, s));
    NR_CUDA_TRY(cudaMemsetAsync(sb + off_wc, 0, off_part - off_wc, s));
    NR_CUDA_TRY(cudaMemcpyAsync(P.wave_count, &one_u, sizeof(one_u), cudaMemcpyHostToDevice, s));
    NR_CUDA_TRY(cudaMemcpyAsync(P.mask[0], root.data(), 16 * W4, cudaMemcpyHostToDevice, s));
    NR_CUDA_TRY(cudaMemcpyAsync(P.mass[0], &one, sizeof(one), cudaMemcpyHostToDevice, s));

    void *args[] = {&P};
    NR_CUDA_TRY(cudaEventRecord(c->ev0, s));
    NR_CUDA_TRY(cudaLaunchCooperativeKernel(kfn, dim3(grid), dim3(block), args, smem, s));
    NR_CUDA_TRY(cudaEventRecord(c->ev1, s));

    std::vector<unsigned long long> wc(max_waves + 1);
    std::vector<NrPartial> parts(grid);
    int status = 0;
    NR_CUDA_TRY(cudaMemcpyAsync(wc.data(), P.wave_count, sizeof(unsigned long long) * wc.size(),
                                cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaMemcpyAsync(parts.data(), P.partials, sizeof(NrPartial) * grid, cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaMemcpyAsync(&status, P.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    NR_CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1));

    NrFix R = nr_fix_zero(), esp = nr_fix_zero();
    unsigned long long nodes = 0, leaves = 0, dead = 0, trunc = 0, spilled = 0;
    for (const NrPartial &p : parts) {          // exact: the order of the additions does not matter
        nr_fix_add(R, p.R);
        nr_fix_add(esp, p.et);
        nr_fix_add(esp, p.es);
        nodes += p.nodes; leaves += p.leaves; dead += p.dead; trunc += p.truncated; spilled += p.spilled;
    }
    int waves = 0;
    unsigned long long maxw = 0;
    for (int k = 0; k <= max_waves; ++k) {
        unsigned long long n = std::min<unsigned long long>(wc[k], cap);
        if (!n) break;
        waves++;
        maxw = std::max(maxw, n);
    }
    r->R = nr_fix_to_double_host(R);
    r->esp = nr_fix_to_double_host(esp);
    r->R_plus_esp = r->R + r->esp;
    r->trunc_bound = r->R > 0 ? r->esp / r->R : r->esp;
    r->nodes = nodes; r->leaves = leaves; r->dead_ends = dead; r->truncated = trunc; r->spilled = spilled;
    r->paths = leaves + spilled;
    r->queued = 0;
    r->iterations = waves;
    r->max_queue_items = maxw;
    r->item_bytes = (int)item_bytes;
    r->max_queue_mb = (double)maxw * item_bytes / (1024.0 * 1024.0);
    r->ms = ms;
    r->time_to_bound_ms = 0;
    r->engine = NR_ENGINE_GRID;
    r->grid_blocks = grid;
    r->block_threads = block;
    r->capacity = cap;
    r->h2d_bytes = blob.size() + sizeof(one_u) + 16 * W4 + sizeof(one);
    r->d2h_bytes = sizeof(unsigned long long) * wc.size() + sizeof(NrPartial) * grid + sizeof(int);
    if (status & NR_DEV_ERR_TIMEOUT) return NR_ERR_TIMEOUT;
    if (status) return NR_ERR_INTERNAL;
    return NR_OK;
}

// ---------------------------------------------------------------------------
// whole-GPU engine for 33..16384 nodes (nr_wide.cuh)
// ---------------------------------------------------------------------------
static void build_wide_blob(const nr_graph *g, int src, int dst, NrWideGraph *wg, std::vector<unsigned char> *blob,
                            const int32_t *terms = nullptr, int nt = 0)
{
    const int n = g->n_nodes, E = g->n_edges;
    const int W = std::max(1, (2 * E + 31) / 32);
    wg->n = n; wg->e = E; wg->w4 = (W + 3) / 4; wg->src = src; wg->dst = dst; wg->n_arcs = g->n_arcs;
    wg->nwd = (n + 31) / 32;
    size_t off = 0;
    wg->off_p = (int)off; off = align16(off + sizeof(double) * std::max(E, 1));
    wg->off_q = (int)off; off = align16(off + sizeof(double) * std::max(E, 1));
    wg->off_row = (int)off; off = align16(off + sizeof(int) * (n + 1));
    wg->off_arc = (int)off; off = align16(off + sizeof(uint32_t) * std::max(g->n_arcs, 1));
    wg->off_kmask = (int)off; off = align16(off + sizeof(uint32_t) * wg->nwd);
    wg->blob_bytes = (int)off;
    blob->assign(off, 0);
    // K-terminal: the terminals other than src
    uint32_t *km = reinterpret_cast<uint32_t *>(blob->data() + wg->off_kmask);
    wg->nk = 0;
    for (int i = 0; i < nt; ++i) {
        const int t = terms[i];
        if (t == src || ((km[t >> 5] >> (t & 31)) & 1u)) continue;
        km[t >> 5] |= 1u << (t & 31);
        wg->nk++;
    }
    double *p = reinterpret_cast<double *>(blob->data() + wg->off_p);
    double *q = reinterpret_cast<double *>(blob->data() + wg->off_q);
    int *row = reinterpret_cast<int *>(blob->data() + wg->off_row);
    uint32_t *arc = reinterpret_cast<uint32_t *>(blob->data() + wg->off_arc);
    for (int e = 0; e < E; ++e) { p[e] = g->edge_p[e]; q[e] = 1.0 - g->edge_p[e]; }
    for (int u = 0; u <= n; ++u) row[u] = g->row_ptr[u];
    for (int j = 0; j < g->n_arcs; ++j)
        arc[j] = ((uint32_t)g->edge_id[j] << NR_WIDE_HEAD_BITS) | (uint32_t)g->col_idx[j];
    wg->tables_global = off > NR_WIDE_STAGE_MAX;
}

static int smem_optin(nr_context *c)
{
    if (!c->smem_optin) {
        int v = 0;
        if (cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device) != cudaSuccess) {
            cudaGetLastError();
            return 48 << 10;
        }
        c->smem_optin = v;
    }
    return c->smem_optin;
}

// Threads of a wide kernel's block: up to NR_WIDE_BLOCK, as many warps as the block's shared
// memory holds (tables, unless read from global memory, and each warp's scratch); 0 if not one.
static int wide_block(nr_context *c, const NrWideGraph &wg)
{
    const size_t lim = (size_t)smem_optin(c);
    for (int w = NR_WIDE_BLOCK / 32; w >= 1; --w)
        if (nr_wide_block_shm(wg, w) <= lim) return 32 * w;
    return 0;
}

static int run_grid_wide(nr_context *c, const nr_graph *g, int src, int dst, uint64_t cap, const nr_options *o,
                         nr_result *r, const int32_t *terms = nullptr, int nt = 0)
{
    c->ckpt.valid = false;                 // the arena is about to be reused
    if (g->n_nodes > NR_WIDE_MAX_N || g->n_edges > 65535) return NR_ERR_UNSUPPORTED;
    NrWideGraph wg;
    std::vector<unsigned char> blob;
    build_wide_blob(g, src, dst, &wg, &blob, terms, nt);
    const int W4 = wg.w4;
    const void *kfn = nr_grid_wide_kernel_ptr(W4);
    if (!kfn) return NR_ERR_UNSUPPORTED;
    const int block = wide_block(c, wg);
    if (!block) return NR_ERR_UNSUPPORTED;
    const size_t smem = nr_wide_block_shm(wg, block / 32);
    NR_CUDA_TRY(nr_smem_limit(c->device, kfn, smem));
    int bps = 0;
    NR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kfn, block, smem));
    if (bps < 1) return NR_ERR_UNSUPPORTED;
    if (o->blocks_per_sm > 0 && o->blocks_per_sm < bps) bps = o->blocks_per_sm;
    const int grid = bps * c->sms;
    const size_t item_bytes = (size_t)W4 * 16 + sizeof(double);
    const size_t mask_bytes = align16((size_t)cap * W4 * 16);
    const size_t mass_bytes = align16((size_t)cap * sizeof(double));
    const size_t qneed = 2 * (mask_bytes + mass_bytes);
    size_t free_b = 0, total_b = 0;
    NR_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    if (qneed > c->qbytes && qneed > free_b + c->qbytes) return NR_ERR_NOMEM;
    int rc = ensure(&c->qbuf, &c->qbytes, qneed);
    if (rc) return rc;
    const int max_waves = g->n_edges + 2;
    size_t off = 0;
    const size_t off_blob = off; off = align16(off + blob.size());
    const size_t off_wc = off; off = align16(off + sizeof(unsigned long long) * (max_waves + 1));
    const size_t off_bar = off; off = align16(off + 4 * sizeof(unsigned));
    const size_t off_part = off; off = align16(off + sizeof(NrPartial) * grid);
    const size_t off_wpart = off; off = align16(off + sizeof(NrWideShare) * 2 * grid);
    const size_t off_stop = off; off = align16(off + 2 * sizeof(int));
    rc = ensure(&c->sbuf, &c->sbytes, off);
    if (rc) return rc;
    unsigned char *sb = static_cast<unsigned char *>(c->sbuf);
    unsigned char *qb = static_cast<unsigned char *>(c->qbuf);
    NrGridWideParams P;
    P.g = wg;
    P.blob = sb + off_blob;
    P.mask[0] = reinterpret_cast<uint4 *>(qb);
    P.mass[0] = reinterpret_cast<double *>(qb + mask_bytes);
    P.mask[1] = reinterpret_cast<uint4 *>(qb + mask_bytes + mass_bytes);
    P.mass[1] = reinterpret_cast<double *>(qb + 2 * mask_bytes + mass_bytes);
    P.capacity = cap;
    P.wave_count = reinterpret_cast<unsigned long long *>(sb + off_wc);
    P.max_waves = max_waves;
    P.bar_count = reinterpret_cast<unsigned *>(sb + off_bar);
    P.bar_gen = P.bar_count + 1;
    P.status = reinterpret_cast<int *>(P.bar_count + 2);
    P.partials = reinterpret_cast<NrPartial *>(sb + off_part);
    P.eps = o->truncation_eps > 0 ? o->truncation_eps : 0.0;
    P.timeout_ns = (long long)((o->timeout_ms > 0 ? o->timeout_ms : 60000.0) * 1e6);
    P.fork = (o->branching == NR_BRANCH_FORK);
    P.border = o->branch_order;
    P.target_on = o->target_width > 0 ? 1 : 0;
    P.target_fix = nr_fix_of(o->target_width > 0 ? o->target_width : 0.0);
    P.max_nodes = o->max_nodes;
    P.wpart = reinterpret_cast<NrWideShare *>(sb + off_wpart);
    P.stop_wave = reinterpret_cast<int *>(sb + off_stop);
    const int stop_init[2] = {-1, 0};
    std::vector<uint32_t> root(4 * W4, 0);
    nr_initial_mask(g, root.data(), 4 * W4);
    const double one = 1.0;
    const unsigned long long one_u = 1;
    cudaStream_t s = c->stream;
    NR_CUDA_TRY(cudaMemcpyAsync(sb + off_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice, s));
    NR_CUDA_TRY(cudaMemsetAsync(sb + off_wc, 0, off_part - off_wc, s));
    NR_CUDA_TRY(cudaMemcpyAsync(P.wave_count, &one_u, sizeof(one_u), cudaMemcpyHostToDevice, s));
    NR_CUDA_TRY(cudaMemcpyAsync(P.mask[0], root.data(), 16 * W4, cudaMemcpyHostToDevice, s));
    NR_CUDA_TRY(cudaMemcpyAsync(P.mass[0], &one, sizeof(one), cudaMemcpyHostToDevice, s));
    NR_CUDA_TRY(cudaMemcpyAsync(P.stop_wave, stop_init, sizeof(stop_init), cudaMemcpyHostToDevice, s));
    void *args[] = {&P};
    NR_CUDA_TRY(cudaEventRecord(c->ev0, s));
    NR_CUDA_TRY(cudaLaunchCooperativeKernel(kfn, dim3(grid), dim3(block), args, smem, s));
    NR_CUDA_TRY(cudaEventRecord(c->ev1, s));
    std::vector<unsigned long long> wc(max_waves + 1);
    std::vector<NrPartial> parts(grid);
    int status = 0;
    NR_CUDA_TRY(cudaMemcpyAsync(wc.data(), P.wave_count, sizeof(unsigned long long) * wc.size(),
                                cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaMemcpyAsync(parts.data(), P.partials, sizeof(NrPartial) * grid, cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaMemcpyAsync(&status, P.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    int stop_out[2] = {-1, 0};
    NR_CUDA_TRY(cudaMemcpyAsync(stop_out, P.stop_wave, sizeof(stop_out), cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    NR_CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    NrFix R = nr_fix_zero(), esp = nr_fix_zero();
    unsigned long long nodes = 0, leaves = 0, dead = 0, trunc = 0, spilled = 0;
    for (const NrPartial &pp : parts) {
        nr_fix_add(R, pp.R);
        nr_fix_add(esp, pp.et);
        nr_fix_add(esp, pp.es);
        nr_fix_add(esp, pp.q);      // still queued at a target stop
        nodes += pp.nodes; leaves += pp.leaves; dead += pp.dead; trunc += pp.truncated; spilled += pp.spilled;
    }
    // waves run (a stop leaves wave stop_wave queued, not run)
    const int stop_wave = stop_out[0];
    int waves = 0;
    unsigned long long maxw = 0, queued = 0;
    const int last = stop_wave >= 0 ? stop_wave : max_waves + 1;
    for (int k = 0; k <= max_waves && k < last; ++k) {
        const unsigned long long nn = std::min<unsigned long long>(wc[k], cap);
        if (!nn) break;
        waves++;
        maxw = std::max(maxw, nn);
    }
    if (stop_wave >= 0) queued = std::min<unsigned long long>(wc[stop_wave], cap);
    r->R = nr_fix_to_double_host(R);
    r->esp = nr_fix_to_double_host(esp);
    r->R_plus_esp = r->R + r->esp;
    r->trunc_bound = r->R > 0 ? r->esp / r->R : r->esp;
    r->nodes = nodes; r->leaves = leaves; r->dead_ends = dead; r->truncated = trunc; r->spilled = spilled;
    r->paths = leaves + spilled;
    r->queued = queued;
    r->stop = stop_wave >= 0 ? stop_out[1] : 0;
    r->iterations = waves;
    r->max_queue_items = maxw;
    r->item_bytes = (int)item_bytes;
    r->max_queue_mb = (double)maxw * item_bytes / (1024.0 * 1024.0);
    r->ms = ms;
    if (stop_wave >= 0 && stop_out[1] == 1) r->time_to_bound_ms = ms;
    r->engine = NR_ENGINE_GRID;
    r->grid_blocks = grid;
    r->block_threads = block;
    r->capacity = cap;
    r->h2d_bytes = blob.size() + sizeof(one_u) + 16 * W4 + sizeof(one) + sizeof(stop_init);
    r->d2h_bytes = sizeof(unsigned long long) * wc.size() + sizeof(NrPartial) * grid + 3 * sizeof(int);
    if (status & NR_DEV_ERR_TIMEOUT) return NR_ERR_TIMEOUT;
    if (status) return NR_ERR_INTERNAL;
    return NR_OK;
}

// Bucket of a mass on the host: the device's nr_bucket (integer operations on the bits).
static int nr_bucket_host(double m, int shift, int nb)
{
    if (shift < 0 || nb <= 1) return 0;
    unsigned long long bits;
    memcpy(&bits, &m, 8);
    long long b = (1023LL << shift) - (long long)(bits >> (52 - shift));
    b = b < 0 ? 0 : b;
    b = b > nb - 1 ? nb - 1 : b;
    return (int)b;
}

// FNV-1a over everything a bucketed run's queue depends on: the graph, the
// terminals, the bucket resolution, eps and the branching.
static uint64_t nr_run_fingerprint(const nr_graph *g, int src, int dst, const nr_options *o)
{
    uint64_t h = 1469598103934665603ull;
    auto mix = [&h](const void *p, size_t n) {
        const unsigned char *b = static_cast<const unsigned char *>(p);
        for (size_t i = 0; i < n; ++i) { h ^= b[i]; h *= 1099511628211ull; }
    };
    mix(&g->n_nodes, sizeof(int32_t)); mix(&g->n_edges, sizeof(int32_t)); mix(&g->n_arcs, sizeof(int32_t));
    mix(g->row_ptr, sizeof(int32_t) * (g->n_nodes + 1));
    mix(g->col_idx, sizeof(int32_t) * g->n_arcs);
    mix(g->edge_id, sizeof(int32_t) * g->n_arcs);
    mix(g->edge_p, sizeof(double) * g->n_edges);
    const int32_t nb = std::max(1, std::min(NR_WIDE_MAX_NB, o->n_buckets > 0 ? (int)o->n_buckets : NR_WIDE_MAX_NB));
    const int32_t v[6] = {src, dst, o->bucket_shift, nb, o->branching, o->branch_order};
    mix(v, sizeof(v));
    const double eps = o->truncation_eps > 0 ? o->truncation_eps : 0.0;
    mix(&eps, sizeof(eps));
    return h;
}

// Whole-GPU bucketed max-mass queue (nr_bucket_wide_kernel) over an arena of
// `cap` slots: 2^shift buckets per factor of two in mass, nb buckets.
static int run_bucket_wide(nr_context *c, const nr_graph *g, int src, int dst, uint64_t cap, const nr_options *o,
                           nr_result *r, const NrResumeIn *rin = nullptr, const int32_t *terms = nullptr,
                           int nt = 0)
{
    if (g->n_nodes > NR_WIDE_MAX_N || g->n_edges > 65535) return NR_ERR_UNSUPPORTED;
    c->ckpt.valid = false;
    const uint64_t live_in = rin ? (uint64_t)rin->mass.size() : 0;
    cap = std::max<uint64_t>(std::max<uint64_t>(64, 2 * live_in),
                             std::min<uint64_t>(cap, 0xffffffffull));   // slot ids are 32-bit
    if (cap > 0xffffffffull) return NR_ERR_UNSUPPORTED;
    const int nb = std::max(1, std::min(NR_WIDE_MAX_NB, o->n_buckets > 0 ? (int)o->n_buckets : NR_WIDE_MAX_NB));
    NrWideGraph wg;
    std::vector<unsigned char> blob;
    build_wide_blob(g, src, dst, &wg, &blob, terms, nt);
    const int W4 = wg.w4;
    const void *kfn = nr_bucket_wide_kernel_ptr(W4);
    if (!kfn) return NR_ERR_UNSUPPORTED;
    const int block = wide_block(c, wg);
    if (!block) return NR_ERR_UNSUPPORTED;
    const size_t smem = nr_wide_block_shm(wg, block / 32);
    NR_CUDA_TRY(nr_smem_limit(c->device, kfn, smem));
    int bps = 0;
    NR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kfn, block, smem));
    if (bps < 1) return NR_ERR_UNSUPPORTED;
    if (o->blocks_per_sm > 0 && o->blocks_per_sm < bps) bps = o->blocks_per_sm;
    const int grid = bps * c->sms;
    const size_t item_bytes = (size_t)W4 * 16 + sizeof(double) + 1;
    // arena: masks, masses, bucket bytes, wave list
    const size_t mask_bytes = align16((size_t)cap * W4 * 16);
    const size_t mass_bytes = align16((size_t)cap * sizeof(double));
    const size_t key_bytes = align16((size_t)cap);
    const size_t list_bytes = align16((size_t)cap * sizeof(unsigned));
    const size_t qneed = mask_bytes + mass_bytes + key_bytes + list_bytes;
    size_t free_b = 0, total_b = 0;
    NR_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    if (qneed > c->qbytes && qneed > free_b + c->qbytes) return NR_ERR_NOMEM;
    int rc = ensure(&c->qbuf, &c->qbytes, qneed);
    if (rc) return rc;
    size_t off = 0;
    const size_t off_blob = off; off = align16(off + blob.size());
    const size_t off_zero = off;                                   // zeroed from here on
    const size_t off_top = off; off = align16(off + sizeof(unsigned long long));
    const size_t off_bc = off; off = align16(off + sizeof(unsigned long long) * nb);
    const size_t off_wl = off; off = align16(off + sizeof(unsigned long long) * 2);
    const size_t off_cc = off; off = align16(off + sizeof(unsigned long long) * 2 * grid);
    const size_t off_bar = off; off = align16(off + 4 * sizeof(unsigned));
    const size_t off_part = off; off = align16(off + sizeof(NrPartial) * grid);
    const size_t off_wpart = off; off = align16(off + sizeof(NrWideShare) * 2 * grid);
    const size_t off_info = off; off = align16(off + 3 * sizeof(int));
    const size_t off_stats = off; off = align16(off + 2 * sizeof(unsigned long long));
    rc = ensure(&c->sbuf, &c->sbytes, off);
    if (rc) return rc;
    unsigned char *sb = static_cast<unsigned char *>(c->sbuf);
    unsigned char *qb = static_cast<unsigned char *>(c->qbuf);
    NrBucketWideParams P;
    P.g = wg;
    P.blob = sb + off_blob;
    P.mask = reinterpret_cast<uint4 *>(qb);
    P.mass = reinterpret_cast<double *>(qb + mask_bytes);
    P.key = qb + mask_bytes + mass_bytes;
    P.list = reinterpret_cast<unsigned *>(qb + mask_bytes + mass_bytes + key_bytes);
    P.capacity = cap;
    P.top = reinterpret_cast<unsigned long long *>(sb + off_top);
    P.bcount = reinterpret_cast<unsigned long long *>(sb + off_bc);
    P.wave_len = reinterpret_cast<unsigned long long *>(sb + off_wl);
    P.ccount = reinterpret_cast<unsigned long long *>(sb + off_cc);
    P.shift = std::max(0, (int)o->bucket_shift);
    P.nb = nb;
    P.max_waves = 1 << 30;
    P.bar_count = reinterpret_cast<unsigned *>(sb + off_bar);
    P.bar_gen = P.bar_count + 1;
    P.status = reinterpret_cast<int *>(P.bar_count + 2);
    P.partials = reinterpret_cast<NrPartial *>(sb + off_part);
    P.eps = o->truncation_eps > 0 ? o->truncation_eps : 0.0;
    P.timeout_ns = (long long)((o->timeout_ms > 0 ? o->timeout_ms : 60000.0) * 1e6);
    P.fork = (o->branching == NR_BRANCH_FORK);
    P.border = o->branch_order;
    P.target_on = o->target_width > 0 ? 1 : 0;
    P.target_fix = nr_fix_of(o->target_width > 0 ? o->target_width : 0.0);
    P.max_nodes = o->max_nodes;
    P.wpart = reinterpret_cast<NrWideShare *>(sb + off_wpart);
    P.stop_info = reinterpret_cast<int *>(sb + off_info);
    P.stats = reinterpret_cast<unsigned long long *>(sb + off_stats);
    P.resume = rin ? 1 : 0;
    P.init_R = P.init_et = P.init_es = P.init_net = nr_fix_zero();
    P.init_nodes = P.init_leaves = P.init_dead = P.init_trunc = P.init_spilled = 0;
    cudaStream_t s = c->stream;
    NR_CUDA_TRY(cudaMemcpyAsync(sb + off_blob, blob.data(), blob.size(), cudaMemcpyHostToDevice, s));
    NR_CUDA_TRY(cudaMemsetAsync(sb + off_zero, 0, off - off_zero, s));
    // host copies must outlive the asynchronous uploads: they live until the synchronise below
    std::vector<unsigned char> keys;
    std::vector<unsigned long long> bcnt;
    NrWideShare share0{};
    unsigned long long top0 = 1;
    if (!rin) {
        // the root: initial mask with mass 1 (main.cu:805-809) in slot 0, bucket 0 (mass 1 is the top bucket)
        std::vector<uint32_t> root(4 * W4, 0);
        nr_initial_mask(g, root.data(), 4 * W4);
        keys.assign(1, 0);
        bcnt.assign(1, 1);
        NR_CUDA_TRY(cudaMemcpy(P.mask, root.data(), 16 * W4, cudaMemcpyHostToDevice));
        const double one = 1.0;
        NR_CUDA_TRY(cudaMemcpy(P.mass, &one, sizeof(one), cudaMemcpyHostToDevice));
    } else {
        // a checkpoint: its records in slots [0, live), their buckets and counts, block 0's sums
        top0 = live_in;
        keys.resize(live_in);
        bcnt.assign(nb, 0);
        for (uint64_t i = 0; i < live_in; ++i) {
            keys[i] = (unsigned char)nr_bucket_host(rin->mass[i], P.shift, nb);
            bcnt[keys[i]]++;
        }
        if (live_in) {
            NR_CUDA_TRY(cudaMemcpy(P.mask, rin->masks.data(), (size_t)live_in * 16 * W4, cudaMemcpyHostToDevice));
            NR_CUDA_TRY(cudaMemcpy(P.mass, rin->mass.data(), (size_t)live_in * sizeof(double),
                                   cudaMemcpyHostToDevice));
        }
        P.init_R = rin->R; P.init_et = rin->et; P.init_es = rin->es; P.init_net = rin->net;
        P.init_nodes = rin->nodes; P.init_leaves = rin->leaves; P.init_dead = rin->dead;
        P.init_trunc = rin->trunc; P.init_spilled = rin->spilled;
        // the shares the first stop test reads (slot 1): block 0 holds the whole width so far
        share0.width = rin->et;
        nr_fix_add(share0.width, rin->es);
        nr_fix_add(share0.width, rin->net);
        share0.nodes = rin->nodes;
    }
    NR_CUDA_TRY(cudaMemcpyAsync(P.top, &top0, sizeof(top0), cudaMemcpyHostToDevice, s));
    NR_CUDA_TRY(cudaMemcpyAsync(P.bcount, bcnt.data(), sizeof(unsigned long long) * bcnt.size(),
                                cudaMemcpyHostToDevice, s));
    if (!keys.empty()) NR_CUDA_TRY(cudaMemcpyAsync(P.key, keys.data(), keys.size(), cudaMemcpyHostToDevice, s));
    if (rin) NR_CUDA_TRY(cudaMemcpyAsync(P.wpart + grid, &share0, sizeof(share0), cudaMemcpyHostToDevice, s));
    void *args[] = {&P};
    NR_CUDA_TRY(cudaEventRecord(c->ev0, s));
    NR_CUDA_TRY(cudaLaunchCooperativeKernel(kfn, dim3(grid), dim3(block), args, smem, s));
    NR_CUDA_TRY(cudaEventRecord(c->ev1, s));
    std::vector<NrPartial> parts(grid);
    int status = 0, info[3] = {0, 0, 0};
    unsigned long long stats[2] = {0, 0};
    NR_CUDA_TRY(cudaMemcpyAsync(parts.data(), P.partials, sizeof(NrPartial) * grid, cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaMemcpyAsync(&status, P.status, sizeof(int), cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaMemcpyAsync(info, P.stop_info, sizeof(info), cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaMemcpyAsync(stats, P.stats, sizeof(stats), cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    NR_CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    NrFix R = nr_fix_zero(), esp = nr_fix_zero(), et = nr_fix_zero(), es = nr_fix_zero(), net = nr_fix_zero();
    unsigned long long nodes = 0, leaves = 0, dead = 0, trunc = 0, spilled = 0;
    for (const NrPartial &pp : parts) {          // exact: the order of the additions does not matter
        nr_fix_add(R, pp.R);
        nr_fix_add(et, pp.et);
        nr_fix_add(es, pp.es);
        nr_fix_add(net, pp.q);                   // still queued
        nodes += pp.nodes; leaves += pp.leaves; dead += pp.dead; trunc += pp.truncated; spilled += pp.spilled;
    }
    esp = et;
    nr_fix_add(esp, es);
    nr_fix_add(esp, net);
    const long long waves_total = (rin ? rin->waves : 0) + info[0];
    const unsigned long long maxw_total = std::max<unsigned long long>(rin ? rin->max_wave : 0, stats[0]);
    if (!status && !(info[0] == P.max_waves) && wg.nk == 0) {   // K-terminal runs are not checkpointed
        NrCkptState &k = c->ckpt;
        k.valid = true;
        k.fp = nr_run_fingerprint(g, src, dst, o);
        k.n = g->n_nodes; k.E = g->n_edges; k.src = src; k.dst = dst; k.W4 = W4;
        k.R = R; k.et = et; k.es = es; k.net = net;
        k.nodes = nodes; k.leaves = leaves; k.dead = dead; k.trunc = trunc; k.spilled = spilled;
        k.max_wave = maxw_total;
        k.waves = waves_total;
        k.cap = cap;
        k.mask_bytes = mask_bytes;
        k.mass_bytes = mass_bytes;
        k.off_top = off_top;
    }
    r->R = nr_fix_to_double_host(R);
    r->esp = nr_fix_to_double_host(esp);
    r->R_plus_esp = r->R + r->esp;
    r->trunc_bound = r->R > 0 ? r->esp / r->R : r->esp;
    r->nodes = nodes; r->leaves = leaves; r->dead_ends = dead; r->truncated = trunc; r->spilled = spilled;
    r->paths = leaves + spilled;
    r->queued = stats[1];
    r->stop = info[1];
    r->iterations = (int)waves_total;
    r->max_queue_items = maxw_total;
    r->item_bytes = (int)item_bytes;
    r->max_queue_mb = (double)maxw_total * item_bytes / (1024.0 * 1024.0);
    r->ms = ms;
    if (info[1] == 1) r->time_to_bound_ms = ms;
    r->engine = NR_ENGINE_GRID;
    r->grid_blocks = grid;
    r->block_threads = block;
    r->capacity = cap;
    r->h2d_bytes = blob.size() + sizeof(top0) + sizeof(unsigned long long) * bcnt.size() + keys.size() +
                   (rin ? live_in * (16 * W4 + sizeof(double)) + sizeof(share0) : 16 * W4 + sizeof(double));
    r->d2h_bytes = sizeof(NrPartial) * grid + sizeof(int) + sizeof(info) + sizeof(stats);
    if (status & NR_DEV_ERR_TIMEOUT) return NR_ERR_TIMEOUT;
    if (status) return NR_ERR_INTERNAL;
    return NR_OK;
}

// 33..16384 nodes: the bucketed max-mass queue for the max-mass order (and for a target width
// in the default order) with a bucket shift >= 0, else breadth-first waves.  The learned
// order is n <= 32 only.
static int run_wide(nr_context *c, const nr_graph *g, int src, int dst, uint64_t capacity, const nr_options *o,
                    nr_result *r, const int32_t *terms = nullptr, int nt = 0)
{
    if (o->order == NR_ORDER_LEARNED) return NR_ERR_UNSUPPORTED;
    const bool buckets = o->bucket_shift >= 0 &&
                         (o->order == NR_ORDER_MAXMASS || (o->order == NR_ORDER_AUTO && o->target_width > 0));
    if (buckets) return run_bucket_wide(c, g, src, dst, capacity ? capacity : (1u << 22), o, r, nullptr, terms, nt);
    return run_grid_wide(c, g, src, dst, capacity ? capacity : (1u << 20), o, r, terms, nt);
}

// ---------------------------------------------------------------------------
// warp-per-instance engine (nr_warp.cuh)
// ---------------------------------------------------------------------------
struct WarpDump {
    float *feat;                     // device buffers (nullptr: no dump)
    uint32_t *mask;
    double *mass;
    int *inst;
    unsigned long long *count;
    unsigned long long cap;
    int stride;
};


static WarpRunCfg warp_cfg(const nr_options *o, uint64_t capacity, bool exhaustive)
{
    WarpRunCfg w;
    w.eps = o->truncation_eps > 0 ? o->truncation_eps : 0.0;
    w.target = o->target_width > 0 ? o->target_width : 0.0;
    if (exhaustive) {
        w.wave_mode = 0; w.shift = -1; w.n_buckets = 32; w.escalate = 1;
        w.max_nodes = o->max_nodes ? o->max_nodes : (1ull << 21);
    } else {
        // NR_ORDER_WAVES: breadth-first waves, i.e. one bucket, whatever bucket_shift says
        w.wave_mode = 1; w.shift = (o->order == NR_ORDER_WAVES) ? -1 : o->bucket_shift;
        w.escalate = 0; w.max_nodes = o->max_nodes;
        w.learned = (o->order == NR_ORDER_LEARNED);
        int nb = o->n_buckets > 0 ? o->n_buckets : 256;
        nb = std::min(1024, (nb + 31) / 32 * 32);
        w.n_buckets = nb;
    }
    w.fork = (o->branching == NR_BRANCH_FORK);
    w.step_cap = (o->test_fault == 2) ? 1 : 0;
    w.border = o->branch_order;
    w.lane = (o->small_kernel != NR_SMALL_GROUP);
    w.lane2 = (o->small_kernel == NR_SMALL_AUTO) && w.wave_mode && w.shift < 0;
    w.lane_slots = (o->lane_slots == 4) ? 4 : 2;
    w.warps_per_block = (o->warps_per_block >= 1 && o->warps_per_block <= NR_WARP_BLOCK_MAX / 32)
                            ? o->warps_per_block : NR_WARP_BLOCK / 32;
    if (capacity == 0) w.pages = o->pages_per_warp > 0 ? std::min(8192, std::max(4, o->pages_per_warp)) : 512;
    else w.pages = (int)std::min<uint64_t>(8192, std::max<uint64_t>(4, (capacity + NR_PAGE - 1) / NR_PAGE));
    return w;
}

static void fill_from_warp(const NrWarpOut &w, const WarpRunCfg &cfg, int W4, nr_result *r)
{
    NrFix esp = w.et;
    nr_fix_add(esp, w.es);
    nr_fix_add(esp, w.q);          // exact pushes - pops: zero on an empty queue
    r->R = nr_fix_to_double_host(w.R);
    r->esp = nr_fix_to_double_host(esp);
    r->R_plus_esp = r->R + r->esp;
    r->trunc_bound = r->R > 0 ? r->esp / r->R : r->esp;
    r->nodes = w.nodes; r->leaves = w.leaves; r->dead_ends = w.dead; r->truncated = w.trunc;
    r->spilled = w.spilled; r->paths = w.leaves + w.spilled; r->queued = w.queued;
    r->iterations = w.waves;
    r->max_queue_items = w.max_wave;
    r->item_bytes = 16 * W4 + 8;
    r->max_queue_mb = (double)w.max_wave * r->item_bytes / (1024.0 * 1024.0);
    r->time_to_bound_ms = w.t_ns / 1e6;
    r->engine = NR_ENGINE_WARP;
    r->stop = w.status;
    r->capacity = (uint64_t)cfg.pages * NR_PAGE;
}

// Solve n instances with the warp engine; instances the engine hands over
// (status 2) are left with engine = 0 for the caller.
static int ensure_host(void **buf, size_t *have, size_t need)
{
    if (*have >= need && *buf) return NR_OK;
    if (*buf) cudaFreeHost(*buf);
    *buf = nullptr;
    *have = 0;
    if (cudaMallocHost(buf, need) != cudaSuccess) {
        cudaGetLastError();
        *buf = nullptr;
        return NR_ERR_NOMEM;
    }
    *have = need;
    return NR_OK;
}

// Solve n instances with the warp engine; instances the engine hands over
// (status 2) are listed in *handover for the caller.  Host work per call:
// one layout pass, a parallel table fill into pinned staging memory, one
// upload, one launch per (group width, mask width) class, one download.
static int slot_ready(NrSlot &sl)
{
    if (sl.stream) return NR_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.ev1);
    if (e != cudaSuccess) {
        nr_last_cuda_error(e, __LINE__, "batch stream set-up");
        return NR_ERR_CUDA;
    }
    return NR_OK;
}

// Build the tables of instances [0, n) of gs on the host and queue their
// upload, the kernels and the read-back of the outputs on slot `sl`.  `base`
// is the index of gs[0] in the caller's batch (for collected children).
static int warp_submit(nr_context *c, NrSlot &sl, int base, int n, const nr_graph *gs, const int32_t *srcs,
                       const int32_t *dsts, const WarpRunCfg &cfg, nr_result *res, PhaseClock &pc,
                       cudaStream_t after = nullptr, bool uniform = false, const double *pmat = nullptr)
{
    constexpr int NCLS = NR_NCLS;
    const bool lane_ok = cfg.lane && !cfg.fork && !cfg.learned && !cfg.dump && cfg.border != NR_BORDER_LEARNED;
    int rc0 = slot_ready(sl);
    if (rc0) return rc0;
    NrBatchScratch &S = sl.scratch;          // kept by the slot: no page faults on every call
    S.desc.resize(n);
    S.cls.resize(n);
    S.same_prev.resize(n);
    S.inst_b.resize(n);
    S.struct_b.resize(n);
    NrSmallGraph *desc = S.desc.data();
    // staging (the same offsets in pinned host memory and on the device):
    //   [work counters | tables (instance order) | descriptors (class order) | ids] then [outputs]
    size_t off_desc = 0, off_ids = 0, up_bytes = 0, off_out = 0;
    const size_t off_cnt = 0;
    int class_count[NCLS] = {0};
    int class_begin[NCLS + 1] = {0};
    unsigned char *hb = nullptr;
    NrSmallGraph *hdesc = nullptr;
    int *hids = nullptr;
    int rc = NR_OK;
    const int B = std::max(1, std::min(NR_HOST_BLOCKS, n / 128));
    auto blk_begin = [&](int b) { return (int)((long long)n * b / B); };
    size_t pm_off = 0, pm_bytes = 0;          // matrix batches: where the matrix goes, its bytes
    if (pmat && !uniform) return NR_ERR_INVALID;
    if (uniform) {
        // one topology (the same CSR arrays) for every instance: every instance's tables have the
        // same size, so the offsets are known without a sizes pass -- instance 0's p, the shared
        // structural part, then the other instances' p -- and one parallel pass validates,
        // describes and copies them.  One class, so class order is instance order.
        int vr = validate_shape(&gs[0], srcs[0], dsts[0]);
        if (!vr) vr = validate_structure(&gs[0]);
        if (vr) return vr;
        NrSmallGraph t;
        const size_t ib = small_inst_layout(&gs[0], srcs[0], dsts[0], &t);
        const size_t sb = small_struct_layout(&gs[0], &t, 0);
        t.rows = rows_mode_of(&gs[0]);
        if (t.w4 > NR_MAX_W4) return NR_ERR_UNSUPPORTED;
        const int G = group_width(gs[0].n_nodes);
        const int cls = (lane_ok && gs[0].n_nodes <= NR_LANE_MAX_N && t.rows == 1 && t.w4 <= NR_LANE_MAX_W4)
                            ? NR_LANE_CLS0 + t.w4 - 1
                            : (G == 8 ? 0 : G == 16 ? 1 : 2) * NR_MAX_W4 + t.w4 - 1;
        size_t off = align16(sizeof(int) * (NCLS + 1));   // work counters, then a NaN flag
        const size_t tbase = off;
        // matrix batches: the structural part, then the caller's matrix as it is (row i =
        // instance i's p; 8-byte rows suffice for the kernels' scalar loads)
        const size_t pm_row = sizeof(double) * (size_t)gs[0].n_edges;
        const size_t off_pm = pmat ? align16(tbase + sb) : 0;
        off = pmat ? align16(off_pm + (size_t)n * pm_row) : align16(off + (size_t)n * ib + sb);
        class_count[cls] = n;
        for (int j = 0; j < NCLS; ++j) class_begin[j + 1] = class_begin[j] + class_count[j];
        off_desc = off; off = align16(off + sizeof(NrSmallGraph) * n);
        off_ids = off; off = align16(off + sizeof(int) * n);
        up_bytes = off;
        off_out = off; off = align16(off + sizeof(NrWarpOut) * n);
        rc = ensure_host(&sl.hbuf, &sl.hbuf_bytes, off);
        if (rc) return rc;
        rc = ensure(&sl.wbuf, &sl.wbuf_bytes, off);
        if (rc) return rc;
        hb = static_cast<unsigned char *>(sl.hbuf);
        hdesc = reinterpret_cast<NrSmallGraph *>(hb + off_desc);
        hids = reinterpret_cast<int *>(hb + off_ids);
        memset(hb + off_cnt, 0, sizeof(int) * (NCLS + 1));
        t.struct_off = (long long)(pmat ? tbase : tbase + ib);
        small_fill_struct(&gs[0], &t, hb + t.struct_off);
        pc.mark("sizes");
        std::atomic<int> bad(NR_OK);
        const int n_nodes0 = gs[0].n_nodes;
        c->parallel_for(B, 1, [&](int b) {
            for (int i = blk_begin(b), e = blk_begin(b + 1); i < e; ++i) {
                NrSmallGraph d = t;
                d.src = srcs[i];
                d.dst = dsts[i];
                if (pmat) {                   // terminals only: the matrix is uploaded as it is
                    if (d.src < 0 || d.dst < 0 || d.src >= n_nodes0 || d.dst >= n_nodes0) {
                        bad.store(NR_ERR_INVALID);
                        continue;
                    }
                    d.blob_off = (long long)(off_pm + (size_t)i * pm_row);
                    d.blob_bytes = (int)pm_row;
                } else {
                    const int v = validate_shape(&gs[i], srcs[i], dsts[i]);
                    if (v) { bad.store(v); continue; }
                    d.blob_off = (long long)(tbase + (i == 0 ? 0 : ib + sb + (size_t)(i - 1) * ib));
                    d.blob_bytes = (int)(ib + (i == 0 ? sb : 0));
                    if (!small_fill_inst(&gs[i], &d, hb + d.blob_off)) bad.store(NR_ERR_INVALID);
                }
                desc[i] = d;
                S.cls[i] = cls;
                hdesc[i] = d;
                hids[i] = i;
            }
        });
        if (bad.load() != NR_OK) return bad.load();
        sl.off_flag = sizeof(int) * NCLS;
        pm_off = off_pm;
        pm_bytes = pmat ? (size_t)n * pm_row : 0;
        pc.mark("tables");
    } else {
    // Host blocks: contiguous instance ranges, one task of the worker pool each.  Two
    // parallel passes (sizes, then offsets and tables) around a serial prefix over blocks.
    S.blk.resize(B);
    std::atomic<int> too_wide(0), invalid(NR_OK);
    c->parallel_for(B, 1, [&](int b) {
        NrHostBlock &k = S.blk[b];
        size_t rel = 0;
        k.last_owner_rel = -1;
        k.last_rows = -1;
        for (int j = 0; j < NCLS; ++j) k.cnt[j] = 0;
        int cur_rows = -1;                    // rows mode of the current topology
        const int i0 = blk_begin(b);
        for (int i = i0, e = blk_begin(b + 1); i < e; ++i) {
            // validation (the shape of every instance; the arrays of the first of a run of
            // instances sharing them, and of the block's first, whose run may start earlier)
            int vr = validate_shape(&gs[i], srcs[i], dsts[i]);
            const bool prev_ok = i > 0 && validate_shape(&gs[i - 1], srcs[i - 1], dsts[i - 1]) == NR_OK;
            if (!vr && (i == i0 || !prev_ok || !same_structure_arrays(&gs[i], &gs[i - 1])))
                vr = validate_structure(&gs[i]);
            if (vr) { invalid.store(vr); S.cls[i] = 0; S.same_prev[i] = 0; S.inst_b[i] = 0; S.struct_b[i] = 0; continue; }
            // consecutive instances with the same topology share one structural part
            const bool same = prev_ok && same_topology(&gs[i], &gs[i - 1]);
            const size_t ib = small_inst_layout(&gs[i], srcs[i], dsts[i], &desc[i]);
            size_t sb = 0;                    // offsets relative to struct_off
            if (same && i > i0) {
                desc[i].off_eid = desc[i - 1].off_eid; desc[i].off_start = desc[i - 1].off_start;
                desc[i].off_list = desc[i - 1].off_list; desc[i].off_rows16 = desc[i - 1].off_rows16;
            } else {
                sb = small_struct_layout(&gs[i], &desc[i], 0);
            }
            S.same_prev[i] = same;
            S.inst_b[i] = ib;
            S.struct_b[i] = same ? 0 : sb;
            rel += ib;
            if (!same) {
                k.last_owner_rel = (long long)rel;
                rel += sb;
                desc[i].rows = rows_mode_of(&gs[i]);
                k.last_rows = desc[i].rows;
                cur_rows = desc[i].rows;
            } else if (cur_rows < 0) {
                cur_rows = rows_mode_of(&gs[i]);   // its owner is in an earlier block
            }
            if (desc[i].w4 > NR_MAX_W4) { too_wide.store(1); S.cls[i] = 0; continue; }
            const int G = group_width(gs[i].n_nodes);
            if (lane_ok && gs[i].n_nodes <= NR_LANE_MAX_N && cur_rows == 1 && desc[i].w4 <= NR_LANE_MAX_W4)
                S.cls[i] = NR_LANE_CLS0 + desc[i].w4 - 1;
            else
                S.cls[i] = (G == 8 ? 0 : G == 16 ? 1 : 2) * NR_MAX_W4 + desc[i].w4 - 1;
            k.cnt[S.cls[i]]++;
        }
        k.bytes = rel;
    });
    if (invalid.load() != NR_OK) return invalid.load();
    if (too_wide.load()) return NR_ERR_UNSUPPORTED;
    pc.mark("sizes");

    size_t off = align16(sizeof(int) * NCLS);
    long long owner_struct = -1;              // struct_off of the last structural part so far
    int owner_rows = 0;                       // and its rows mode
    for (int b = 0; b < B; ++b) {
        NrHostBlock &k = S.blk[b];
        k.base = off;
        k.struct_in = owner_struct;
        k.rows_in = owner_rows;
        if (k.last_owner_rel >= 0) owner_struct = (long long)off + k.last_owner_rel;
        if (k.last_rows >= 0) owner_rows = k.last_rows;
        off += k.bytes;
        for (int j = 0; j < NCLS; ++j) {
            k.cbase[j] = class_count[j];
            class_count[j] += k.cnt[j];
        }
    }
    for (int j = 0; j < NCLS; ++j) class_begin[j + 1] = class_begin[j] + class_count[j];
    off = align16(off);
    off_desc = off; off = align16(off + sizeof(NrSmallGraph) * n);
    off_ids = off; off = align16(off + sizeof(int) * n);
    up_bytes = off;
    off_out = off; off = align16(off + sizeof(NrWarpOut) * n);
    rc = ensure_host(&sl.hbuf, &sl.hbuf_bytes, off);
    if (rc) return rc;
    rc = ensure(&sl.wbuf, &sl.wbuf_bytes, off);
    if (rc) return rc;
    hb = static_cast<unsigned char *>(sl.hbuf);
    hdesc = reinterpret_cast<NrSmallGraph *>(hb + off_desc);
    hids = reinterpret_cast<int *>(hb + off_ids);
    memset(hb + off_cnt, 0, sizeof(int) * NCLS);
    std::atomic<int> bad_p(0);            // a NaN probability
    c->parallel_for(B, 1, [&](int b) {
        const NrHostBlock &k = S.blk[b];
        size_t at = k.base;
        long long rep = k.struct_in;
        int rep_rows = k.rows_in;
        int fill[NCLS];
        for (int j = 0; j < NCLS; ++j) fill[j] = class_begin[j] + k.cbase[j];
        for (int i = blk_begin(b), e = blk_begin(b + 1); i < e; ++i) {
            NrSmallGraph &d = desc[i];
            d.blob_off = (long long)at;
            at += S.inst_b[i];
            if (!S.same_prev[i]) {
                d.struct_off = (long long)at;
                rep = d.struct_off;
                rep_rows = d.rows;
                at += S.struct_b[i];
                small_fill_struct(&gs[i], &d, hb + d.struct_off);
            } else {
                d.struct_off = rep;               // instance 0 always owns one, so rep >= 0 here
                d.rows = rep_rows;
            }
            d.blob_bytes = (int)(S.inst_b[i] + S.struct_b[i]);
            if (!small_fill_inst(&gs[i], &d, hb + d.blob_off)) bad_p.store(1);
            const int slot = fill[S.cls[i]]++;
            hdesc[slot] = d;
            hids[slot] = i;
        }
    });
    if (bad_p.load()) return NR_ERR_INVALID;
    pc.mark("tables");
    }

    // launch geometry per class (occupancy cached per kernel and shared-memory size)
    const int warps_pb = cfg.warps_per_block, block = 32 * warps_pb;
    if (!c->smem_optin) {
        int v = 0;
        NR_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
        c->smem_optin = v;
    }
    // pages per warp: as asked, but no more than the block's shared memory can index
    WarpRunCfg cfgp = cfg;
    while (cfgp.pages > 4 &&
           std::max(std::max(nr_warp_shm_bytes(4, NR_MAX_W4, cfgp.n_buckets, cfgp.pages, true),
                             nr_lane_shm_bytes(cfgp.n_buckets, cfgp.pages)),
                    nr_lane2_shm_bytes(cfgp.pages, cfg.lane_slots)) * warps_pb > (size_t)c->smem_optin)
        cfgp.pages /= 2;
    const bool learn = cfg.learned || cfg.dump || cfg.border == NR_BORDER_LEARNED;
    int grids[NCLS] = {0};
    size_t smems[NCLS] = {0};
    size_t slab_need = 0;
    for (int j = 0; j < NCLS; ++j) {
        if (!class_count[j]) continue;
        const bool lanek = j >= NR_LANE_CLS0;
        const int G = lanek ? 0 : 8 << (j / NR_MAX_W4);
        const int W4 = lanek ? j - NR_LANE_CLS0 + 1 : j % NR_MAX_W4 + 1;
        const bool two = lanek && cfg.lane2;
        const void *kfn = lanek ? (two ? nr_lane2_kernel_ptr(W4, cfg.lane_slots) : nr_lane_kernel_ptr(W4))
                                : warp_kernel(G, W4, learn, cfg.fork != 0);
        if (!kfn) return NR_ERR_UNSUPPORTED;
        const size_t smem = (two ? nr_lane2_shm_bytes(cfgp.pages, cfg.lane_slots)
                                 : lanek ? nr_lane_shm_bytes(cfg.n_buckets, cfgp.pages)
                                         : nr_warp_shm_bytes(32 / G, W4, cfg.n_buckets, cfgp.pages, learn)) * warps_pb;
        auto it = c->occupancy.find({kfn, smem * 64 + warps_pb});
        int bps;
        if (it == c->occupancy.end()) {
            NR_CUDA_TRY(nr_smem_limit(c->device, kfn, smem));
            NR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kfn, block, smem));
            c->occupancy[{kfn, smem * 64 + warps_pb}] = bps;
        } else {
            bps = it->second;
        }
        if (bps < 1) return NR_ERR_UNSUPPORTED;
        const int per_block = warps_pb * (two ? cfg.lane_slots : 1);   // instances a block starts with
        grids[j] = std::max(1, std::min(bps * c->sms, (class_count[j] + per_block - 1) / per_block));
        smems[j] = smem;
        const size_t row_bytes = lanek ? 4 * (size_t)NR_LANE_ROW_WORDS : 4 * (size_t)G;
        slab_need = std::max(slab_need, (size_t)grids[j] * warps_pb * cfgp.pages * NR_PAGE *
                                            (16 * (size_t)W4 + 8 + row_bytes));
    }
    rc = ensure(&sl.wslab, &sl.wslab_bytes, slab_need);
    if (rc) return rc;
    unsigned char *wb = static_cast<unsigned char *>(sl.wbuf);
    cudaStream_t s = sl.stream;
    pc.mark("geometry");
    if (after) {                          // the upload waits for the caller's stream
        if (!c->ev_after) NR_CUDA_TRY(cudaEventCreateWithFlags(&c->ev_after, cudaEventDisableTiming));
        NR_CUDA_TRY(cudaEventRecord(c->ev_after, after));
        NR_CUDA_TRY(cudaStreamWaitEvent(s, c->ev_after, 0));
    }
    if (pmat) {
        // counters and structural part, the caller's matrix straight from its memory (a plain DMA
        // when it is pinned), descriptors and ids; then a scan of the matrix for NaN on the device
        NR_CUDA_TRY(cudaMemcpyAsync(wb, hb, pm_off, cudaMemcpyHostToDevice, s));
        NR_CUDA_TRY(cudaMemcpyAsync(wb + pm_off, pmat, pm_bytes, cudaMemcpyHostToDevice, s));
        NR_CUDA_TRY(cudaMemcpyAsync(wb + off_desc, hb + off_desc, up_bytes - off_desc, cudaMemcpyHostToDevice, s));
        NR_CUDA_TRY(nr_launch_nan_scan(reinterpret_cast<const double *>(wb + pm_off), pm_bytes / sizeof(double),
                                       reinterpret_cast<int *>(wb + sl.off_flag), s));
    } else {
        NR_CUDA_TRY(cudaMemcpyAsync(wb, hb, up_bytes, cudaMemcpyHostToDevice, s));
    }
    NR_CUDA_TRY(cudaEventRecord(sl.ev0, s));
    int first_grid = 0;
    for (int j = 0; j < NCLS; ++j) {
        if (!class_count[j]) continue;
        const bool lanek = j >= NR_LANE_CLS0;
        const int G = lanek ? 0 : 8 << (j / NR_MAX_W4);
        const int W4 = lanek ? j - NR_LANE_CLS0 + 1 : j % NR_MAX_W4 + 1;
        if (!first_grid) first_grid = grids[j];
        NrWarpParams P;
        P.blob = wb;
        P.inst = reinterpret_cast<const NrSmallGraph *>(wb + off_desc) + class_begin[j];
        P.inst_id = reinterpret_cast<const int *>(wb + off_ids) + class_begin[j];
        P.n_inst = class_count[j];
        P.next_inst = reinterpret_cast<int *>(wb + off_cnt) + j;
        P.slab_mask = static_cast<uint4 *>(sl.wslab);
        const size_t warps = (size_t)grids[j] * warps_pb;
        P.slab_mass = reinterpret_cast<double *>(static_cast<unsigned char *>(sl.wslab) +
                                                 warps * cfgp.pages * NR_PAGE * 16 * (size_t)W4);
        P.slab_rows = reinterpret_cast<uint32_t *>(static_cast<unsigned char *>(sl.wslab) +
                                                   warps * cfgp.pages * NR_PAGE * (16 * (size_t)W4 + 8));
        P.pages = cfgp.pages;
        P.n_buckets = cfg.n_buckets;
        P.shift = cfg.shift;
        P.wave_mode = cfg.wave_mode;
        P.escalate = cfg.escalate;
        P.eps = cfg.eps;
        P.target = cfg.target;
        P.target_fix = nr_fix_of(cfg.target);
        P.max_nodes = cfg.max_nodes;
        P.out = reinterpret_cast<NrWarpOut *>(wb + off_out);
        P.learned = cfg.learned;
        P.mlp = c->mlp;
        P.dump_feat = cfg.dump ? cfg.dump->feat : nullptr;
        P.dump_mask = cfg.dump ? cfg.dump->mask : nullptr;
        P.dump_mass = cfg.dump ? cfg.dump->mass : nullptr;
        P.dump_inst = cfg.dump ? cfg.dump->inst : nullptr;
        P.dump_count = cfg.dump ? cfg.dump->count : nullptr;
        P.dump_cap = cfg.dump ? cfg.dump->cap : 0;
        P.dump_stride = cfg.dump ? cfg.dump->stride : 0;
        P.inst_base = base;
        P.fork = cfg.fork;
        P.step_cap = cfg.step_cap;
        P.border = cfg.border;
        const void *kfn = lanek ? (cfg.lane2 ? nr_lane2_kernel_ptr(W4, cfg.lane_slots) : nr_lane_kernel_ptr(W4))
                                : warp_kernel(G, W4, learn, cfg.fork != 0);
        void *args[] = {&P};
        NR_CUDA_TRY(nr_smem_limit(c->device, kfn, smems[j]));
        NR_CUDA_TRY(cudaLaunchKernel(kfn, dim3(grids[j]), dim3(block), args, smems[j], s));
    }
    NR_CUDA_TRY(cudaEventRecord(sl.ev1, s));
    NrWarpOut *hout = reinterpret_cast<NrWarpOut *>(hb + off_out);
    NR_CUDA_TRY(cudaMemcpyAsync(hout, wb + off_out, sizeof(NrWarpOut) * n, cudaMemcpyDeviceToHost, s));
    if (pmat) NR_CUDA_TRY(cudaMemcpyAsync(hb + sl.off_flag, wb + sl.off_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    sl.matrix = (pmat != nullptr);
    sl.pmat = pmat;
    sl.n = n; sl.gs = gs; sl.srcs = srcs; sl.dsts = dsts; sl.res = res;
    sl.cfgp = cfgp; sl.off_out = off_out; sl.first_grid = first_grid; sl.block = block;
    pc.mark("enqueue");
    return NR_OK;
}

// Wait for the part queued on slot `sl` and fill its results; instances the
// warp engine handed over are appended to `handover` (plus `base`).
static int warp_finish(nr_context *c, NrSlot &sl, int base, std::vector<int> *handover, PhaseClock &pc)
{
    NR_CUDA_TRY(cudaStreamSynchronize(sl.stream));
    pc.mark("device");
    float ms = 0.f;
    NR_CUDA_TRY(cudaEventElapsedTime(&ms, sl.ev0, sl.ev1));
    const int n = sl.n;
    const nr_graph *gs = sl.gs;
    const NrSmallGraph *desc = sl.scratch.desc.data();
    const NrWarpOut *hout = reinterpret_cast<const NrWarpOut *>(static_cast<unsigned char *>(sl.hbuf) + sl.off_out);
    if (sl.matrix && *reinterpret_cast<const int *>(static_cast<unsigned char *>(sl.hbuf) + sl.off_flag))
        return NR_ERR_INVALID;                // a NaN probability in the caller's matrix
    const int gstride = sl.matrix ? 0 : 1;    // matrix batches: one topology for every instance
    std::atomic<int> n_hand(0), n_check(0);
    c->parallel_for(n, 256, [&](int i) {
        nr_result *r = &sl.res[i];
        memset(r, 0, sizeof(*r));
        const nr_graph &gi = gs[i * gstride];
        r->n_nodes = gi.n_nodes; r->n_edges = gi.n_edges; r->src = sl.srcs[i]; r->dst = sl.dsts[i];
        r->mask_words = std::max(1, (2 * gi.n_edges + 31) / 32);
        if (hout[i].status == 2) { n_hand.fetch_add(1); return; }
        if (hout[i].status == NR_LANE_STATUS_CHECK) { n_check.fetch_add(1); return; }
        fill_from_warp(hout[i], sl.cfgp, desc[i].w4, r);
        r->kernel = sl.scratch.cls[i] < NR_LANE_CLS0 ? NR_KERNEL_GROUP
                    : sl.cfgp.lane2 ? NR_KERNEL_LANE2 : NR_KERNEL_LANE;
        r->ms = ms;
        r->grid_blocks = sl.first_grid;
        r->block_threads = sl.block;
        r->h2d_bytes = desc[i].blob_bytes + sizeof(NrSmallGraph) + sizeof(int);
        r->d2h_bytes = sizeof(NrWarpOut);
    });
    if (n_check.load()) {
        for (int i = 0; i < n; ++i)
            if (hout[i].status == NR_LANE_STATUS_CHECK) {
                snprintf(g_internal, sizeof(g_internal), "warp engine check %llu failed on instance %d",
                         (unsigned long long)hout[i].max_wave, base + i);
                break;
            }
        return NR_ERR_INTERNAL;
    }
    if (n_hand.load())
        for (int i = 0; i < n; ++i)
            if (hout[i].status == 2) handover->push_back(base + i);
    pc.mark("results");
    return NR_OK;
}

// Warp engine over instances [0, n) on slot 0.
static int run_warp_batch(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                          const WarpRunCfg &cfg, nr_result *res, std::vector<int> *handover,
                          PhaseClock *clock = nullptr)
{
    PhaseClock local;
    PhaseClock &pc = clock ? *clock : local;
    int rc = warp_submit(c, c->slot[0], 0, n, gs, srcs, dsts, cfg, res, pc);
    if (rc) return rc;
    return warp_finish(c, c->slot[0], 0, handover, pc);
}

// Checks of a batch: shapes, CSR arrays (once per run of instances sharing them),
// probabilities of graphs above 32 nodes (the warp engine checks its own while
// copying them).  *n_wide = graphs above 32 nodes.
// The branch order: a known value; the learned one needs a model and runs on the warp engine
// only (a target width or a max-mass / learned order, path branching).
static int branch_order_ok(const nr_context *c, const nr_options &o)
{
    if (o.branch_order < NR_BORDER_SRC || o.branch_order > NR_BORDER_LEARNED) return NR_ERR_INVALID;
    if (o.branch_order != NR_BORDER_LEARNED) return NR_OK;
    if (!c->has_model) return NR_ERR_INVALID;
    if (o.branching != NR_BRANCH_PATH) return NR_ERR_UNSUPPORTED;
    if (!(o.target_width > 0) && o.order != NR_ORDER_MAXMASS && o.order != NR_ORDER_LEARNED) return NR_ERR_UNSUPPORTED;
    return NR_OK;
}

static int batch_options_ok(const nr_context *c, const nr_options &o)
{
    if (o.order == NR_ORDER_LEARNED && !c->has_model) return NR_ERR_INVALID;
    if (const int rb = branch_order_ok(c, o)) return rb;
    if (o.order == NR_ORDER_LEARNED && o.branching == NR_BRANCH_FORK) return NR_ERR_UNSUPPORTED;
    if (o.branching != NR_BRANCH_PATH && o.branching != NR_BRANCH_FORK) return NR_ERR_INVALID;
    return NR_OK;
}

static int batch_validate(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                          const nr_options &o, int *n_wide)
{
    std::atomic<int> bad(NR_OK), wide(0);
    c->parallel_for(n, 256, [&](int i) {
        int rc = validate_shape(&gs[i], srcs[i], dsts[i]);
        if (!rc && !(i > 0 && same_structure_arrays(&gs[i], &gs[i - 1]))) rc = validate_structure(&gs[i]);
        if (!rc && gs[i].n_nodes > NR_SMALL_MAX_N) {
            rc = validate_probabilities(&gs[i]);
            if (!rc && (o.order == NR_ORDER_LEARNED || o.branch_order == NR_BORDER_LEARNED))
                rc = NR_ERR_UNSUPPORTED;    // learned order and branch order: n <= 32 only
            wide.fetch_add(1);
        }
        if (rc) bad.store(rc);
    });
    *n_wide = wide.load();
    if (bad.load() != NR_OK) return bad.load();
    return batch_options_ok(c, o);
}

static WarpRunCfg batch_cfg(const nr_options &o, uint64_t capacity)
{
    const bool exhaustive = !(o.target_width > 0) && o.order != NR_ORDER_MAXMASS && o.order != NR_ORDER_LEARNED;
    return warp_cfg(&o, capacity, exhaustive);
}

// Instances the warp engine handed over (exhaustive runs that outgrew a warp's
// budget) finish on the whole-GPU engine.
static int run_handover(nr_context *c, const std::vector<int> &handover, const nr_graph *gs, const int32_t *srcs,
                        const int32_t *dsts, uint64_t capacity, const nr_options &o, nr_result *res,
                        const double *pmat = nullptr)
{
    for (int i : handover) {
        nr_graph gi = pmat ? gs[0] : gs[i];      // matrix batches: the topology with row i of the matrix
        if (pmat) gi.edge_p = pmat + (size_t)i * gi.n_edges;
        const int rc = run_grid_small(c, &gi, srcs[i], dsts[i], std::max<uint64_t>(capacity, 1u << 22), &o, &res[i]);
        if (rc) return rc;
    }
    return NR_OK;
}

// A batch with graphs above 32 nodes, start to end: graphs of up to 32 nodes run
// together on the warp engine, larger ones one at a time on the whole-GPU engine.
static int run_mixed_batch(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                           uint64_t capacity, const nr_options &o, nr_result *res)
{
    std::vector<int> small_idx, wide_idx, handover;
    for (int i = 0; i < n; ++i) (gs[i].n_nodes > NR_SMALL_MAX_N ? wide_idx : small_idx).push_back(i);
    int rc;
    if (!small_idx.empty()) {
        const int m = (int)small_idx.size();
        std::vector<nr_graph> sg(m);
        std::vector<int32_t> ss(m), sd(m);
        std::vector<nr_result> sr(m);
        for (int k = 0; k < m; ++k) {
            sg[k] = gs[small_idx[k]]; ss[k] = srcs[small_idx[k]]; sd[k] = dsts[small_idx[k]];
        }
        std::vector<int> hk;
        rc = run_warp_batch(c, m, sg.data(), ss.data(), sd.data(), batch_cfg(o, capacity), sr.data(), &hk);
        if (rc) return rc;
        for (int k = 0; k < m; ++k) res[small_idx[k]] = sr[k];
        for (int k : hk) handover.push_back(small_idx[k]);
    }
    rc = run_handover(c, handover, gs, srcs, dsts, capacity, o, res);
    if (rc) return rc;
    for (int i : wide_idx) {
        nr_result *r = &res[i];
        memset(r, 0, sizeof(*r));
        r->n_nodes = gs[i].n_nodes; r->n_edges = gs[i].n_edges; r->src = srcs[i]; r->dst = dsts[i];
        r->mask_words = std::max(1, (2 * gs[i].n_edges + 31) / 32);
        rc = run_wide(c, &gs[i], srcs[i], dsts[i], std::max<uint64_t>(capacity, 1u << 22), &o, r);
        if (rc) return rc;
    }
    return NR_OK;
}

// Finish the batch queued on a slot: results, then handed-over instances.
static int slot_finish(nr_context *c, NrSlot &sl)
{
    PhaseClock pc;
    std::vector<int> handover;
    sl.pending = false;
    int rc = warp_finish(c, sl, 0, &handover, pc);
    if (!rc) rc = run_handover(c, handover, sl.gs, sl.srcs, sl.dsts, sl.capacity, sl.opt, sl.res,
                               sl.matrix ? sl.pmat : nullptr);
    return rc;
}

// Finish every batch still in flight (before work that uses slot 0 or swaps the model);
// their statuses wait for their tickets.
static void drain(nr_context *c)
{
    for (NrSlot &sl : c->slot)
        if (sl.pending) c->done_rc[sl.ticket] = slot_finish(c, sl);
}

static void record_done(nr_context *c, int64_t ticket, int rc)
{
    c->done_rc[ticket] = rc;
    while (c->done_rc.size() > 64) c->done_rc.erase(c->done_rc.begin());    // waits never made
}

extern "C" int nr_batch_submit(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                               uint64_t capacity, const nr_options *opt, nr_result *res, void *after_stream,
                               int64_t *ticket)
{
    if (!c || !ticket || n < 0 || (n > 0 && (!gs || !srcs || !dsts || !res))) return NR_ERR_INVALID;
    nr_options o;
    if (opt) o = *opt; else nr_options_default(&o);
    std::lock_guard<std::mutex> lock(c->mu);
    const int64_t t = c->next_ticket++;
    *ticket = t;
    if (n == 0) { record_done(c, t, NR_OK); return NR_OK; }
    PhaseClock pc;
    // graphs of up to 32 nodes only (the usual batch): the warp engine's first host pass
    // validates them as it sizes their tables; else the whole batch is validated here first
    bool any_wide = false, uniform = true;   // uniform: one topology (the same CSR arrays) throughout
    for (int i = 0; i < n && !any_wide; ++i) {
        any_wide = gs[i].n_nodes > NR_SMALL_MAX_N;
        uniform = uniform && same_structure_arrays(&gs[i], &gs[0]);
    }
    int n_wide = 0;
    int rc = any_wide ? batch_validate(c, n, gs, srcs, dsts, o, &n_wide) : batch_options_ok(c, o);
    if (rc) { record_done(c, t, rc); return rc; }
    pc.mark("validate");
    NR_CUDA_TRY(cudaSetDevice(c->device));
    if (n_wide) {                             // larger graphs: the whole batch now
        drain(c);
        rc = run_mixed_batch(c, n, gs, srcs, dsts, capacity, o, res);
        record_done(c, t, rc);
        return rc;
    }
    NrSlot &sl = c->slot[(t - 1) % NR_SLOTS];
    if (sl.pending) record_done(c, sl.ticket, slot_finish(c, sl));
    rc = warp_submit(c, sl, 0, n, gs, srcs, dsts, batch_cfg(o, capacity), res, pc,
                     static_cast<cudaStream_t>(after_stream), uniform);
    if (rc) {
        cudaStreamSynchronize(sl.stream);
        record_done(c, t, rc);
        return rc;
    }
    sl.ticket = t;
    sl.pending = true;
    sl.capacity = capacity;
    sl.opt = o;
    return NR_OK;
}

extern "C" int nr_batch_wait(nr_context *c, int64_t ticket)
{
    if (!c) return NR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(c->mu);
    for (NrSlot &sl : c->slot)
        if (sl.pending && sl.ticket == ticket) {
            NR_CUDA_TRY(cudaSetDevice(c->device));
            return slot_finish(c, sl);
        }
    auto it = c->done_rc.find(ticket);
    if (it == c->done_rc.end()) return NR_ERR_INVALID;
    const int rc = it->second;
    c->done_rc.erase(it);
    return rc;
}

// One topology, a matrix of probability sets (nr.h): the topology is checked once, the
// terminals per instance, the matrix for NaN on the device; no per-instance host tables.
extern "C" int nr_batch_submit_matrix(nr_context *c, const nr_graph *topo, int n, const double *p_matrix,
                                      const int32_t *srcs, const int32_t *dsts, uint64_t capacity,
                                      const nr_options *opt, nr_result *res, void *after_stream, int64_t *ticket)
{
    if (!c || !ticket || !topo || n < 0 || (n > 0 && (!p_matrix || !srcs || !dsts || !res))) return NR_ERR_INVALID;
    nr_options o;
    if (opt) o = *opt; else nr_options_default(&o);
    std::lock_guard<std::mutex> lock(c->mu);
    const int64_t t = c->next_ticket++;
    *ticket = t;
    if (n == 0) { record_done(c, t, NR_OK); return NR_OK; }
    int rc = validate_shape(topo, srcs[0], dsts[0]);
    if (!rc) rc = validate_structure(topo);
    if (!rc && topo->n_nodes > NR_SMALL_MAX_N) rc = NR_ERR_UNSUPPORTED;
    if (!rc) rc = batch_options_ok(c, o);
    if (rc) { record_done(c, t, rc); return rc; }
    NR_CUDA_TRY(cudaSetDevice(c->device));
    PhaseClock pc;
    NrSlot &sl = c->slot[(t - 1) % NR_SLOTS];
    if (sl.pending) record_done(c, sl.ticket, slot_finish(c, sl));
    rc = warp_submit(c, sl, 0, n, topo, srcs, dsts, batch_cfg(o, capacity), res, pc,
                     static_cast<cudaStream_t>(after_stream), true, p_matrix);
    if (rc) {
        cudaStreamSynchronize(sl.stream);
        sl.matrix = false;
        record_done(c, t, rc);
        return rc;
    }
    sl.ticket = t;
    sl.pending = true;
    sl.capacity = capacity;
    sl.opt = o;
    return NR_OK;
}

extern "C" int nr_reliability_batch_matrix(nr_context *c, const nr_graph *topo, int n, const double *p_matrix,
                                           const int32_t *srcs, const int32_t *dsts, uint64_t capacity,
                                           const nr_options *opt, nr_result *res)
{
    int64_t t = 0;
    const int rc = nr_batch_submit_matrix(c, topo, n, p_matrix, srcs, dsts, capacity, opt, res, nullptr, &t);
    if (rc) return rc;
    return nr_batch_wait(c, t);
}

extern "C" int nr_reliability_batch(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs,
                                    const int32_t *dsts, uint64_t capacity, const nr_options *opt,
                                    nr_result *res)
{
    if (!c || n < 0 || (n > 0 && (!gs || !srcs || !dsts || !res))) return NR_ERR_INVALID;
    int64_t t = 0;
    const int rc = nr_batch_submit(c, n, gs, srcs, dsts, capacity, opt, res, nullptr, &t);
    const int rw = nr_batch_wait(c, t);
    return rc ? rc : rw;
}

// Autotuner: time candidate warp-engine settings on (a sample of) the batch
// and return the fastest.  Candidates: bucket resolution (2^shift buckets per
// octave, shift 0..2, or one bucket = breadth-first waves; the "bucket count"), pages per warp (the pop chunk:
// how much of a bucket a warp holds and takes at a time), and warps per
// block.  Every candidate gives a valid result (exact counts for exhaustive
// runs; for truncated runs a bracket whose width meets the target); the
// choice only changes time, and for truncated runs where the stop falls.
extern "C" int nr_autotune(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                           uint64_t capacity, const nr_options *opt, nr_options *best, double *best_ms)
{
    if (!c || n <= 0 || !gs || !srcs || !dsts || !best) return NR_ERR_INVALID;
    nr_options base;
    if (opt) base = *opt; else nr_options_default(&base);
    const int sample = std::min(n, 4096);
    std::vector<nr_result> res(sample);
    const bool exhaustive = !(base.target_width > 0) && base.order != NR_ORDER_MAXMASS &&
                            base.order != NR_ORDER_LEARNED;
    // The bucket resolution is searched only when the caller leaves the order to the engine:
    // NR_ORDER_WAVES holds one bucket (breadth-first waves), NR_ORDER_MAXMASS the caller's shift.
    const int shifts_t[] = {-1, 0, 1, 2};   // -1: one bucket, i.e. breadth-first waves
    const int shifts_e[] = {base.order == NR_ORDER_WAVES ? -1 : base.bucket_shift};
    const bool held = exhaustive || base.order == NR_ORDER_WAVES || base.order == NR_ORDER_MAXMASS ||
                      base.order == NR_ORDER_LEARNED;
    const int *shifts = held ? shifts_e : shifts_t;
    const int n_shift = held ? 1 : 4;
    // pages per warp: 64 and 512 (small and medium queues), 4096 for instances whose waves
    // outgrow 512 pages; with a capacity, candidates above it collapse onto it
    const uint64_t pages_c[] = {64, 512, 4096};
    const int wpb_c[] = {2, 4, 8};
    // A candidate is ranked by the instances whose queue spilled (a spill widens the bracket, so
    // fewer is better whatever the time), then by device time: the best of three runs, and for
    // the three leaders three more after every candidate has run once (clock and cache state
    // drift over a search).
    struct Cand { nr_options o; uint64_t cap; int spills; double t; };
    std::vector<Cand> cands;
    auto time_it = [&](Cand &k, int reps) -> int {
        for (int rep = 0; rep < reps; ++rep) {
            int rc = nr_reliability_batch(c, sample, gs, srcs, dsts, k.cap, &k.o, res.data());
            if (rc) return rc;
            double ms = 0;
            bool warp_only = true;
            int spills = 0;
            for (int i = 0; i < sample; ++i) {
                if (res[i].engine != NR_ENGINE_WARP) warp_only = false;
                spills += res[i].spilled != 0;
                ms = std::max(ms, res[i].ms);
            }
            if (!warp_only) ms = 1e300;      // a hand-over costs a full extra solve
            k.t = std::min(k.t, ms);
            k.spills = spills;
        }
        return NR_OK;
    };
    for (int si = 0; si < n_shift; ++si)
        for (int pi = 0; pi < 3; ++pi)
            for (int wpb : wpb_c) {
                const uint64_t pg = pages_c[pi];
                if (pi > 0 && capacity && capacity <= pages_c[pi - 1] * NR_PAGE) continue;
                Cand k;
                k.o = base;
                k.o.bucket_shift = shifts[si];
                k.o.n_buckets = held && base.n_buckets > 0 ? base.n_buckets : 64 << std::max(0, shifts[si]);
                k.o.warps_per_block = wpb;
                k.o.max_nodes = base.max_nodes;
                // the queue size timed: pages_per_warp applies to calls with capacity 0
                k.o.pages_per_warp = (int32_t)std::min<uint64_t>(pg, capacity ? (capacity + NR_PAGE - 1) / NR_PAGE : pg);
                k.cap = capacity ? std::min<uint64_t>(capacity, pg * NR_PAGE) : pg * NR_PAGE;
                k.spills = 0;
                k.t = 1e300;
                const int rc = time_it(k, 3);
                if (rc) return rc;
                cands.push_back(k);
            }
    auto better = [](const Cand &a, const Cand &b) { return a.spills != b.spills ? a.spills < b.spills : a.t < b.t; };
    std::sort(cands.begin(), cands.end(), better);
    for (size_t i = 0; i < std::min<size_t>(3, cands.size()); ++i) {
        const int rc = time_it(cands[i], 3);
        if (rc) return rc;
    }
    std::sort(cands.begin(), cands.begin() + std::min<size_t>(3, cands.size()), better);
    *best = cands[0].o;
    if (best_ms) *best_ms = cands[0].t;
    return NR_OK;
}

// Install the learned scorer's parameters (flat FP32, nr_mlp_param_count()
// floats) on the context; NR_ORDER_LEARNED calls use its BF16 copy.
extern "C" int nr_context_set_model(nr_context *c, const float *params)
{
    if (!c || !params) return NR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(c->mu);
    drain(c);                          // finish batches in flight: slot 0 and the model are used here
    NR_CUDA_TRY(cudaSetDevice(c->device));
    int rc = nr_mlp_upload(params, &c->model, &c->mlp, c->stream);
    if (rc) return rc;
    NR_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->has_model = true;
    return NR_OK;
}

// Solve a batch with the warp engine (options as nr_reliability_batch) and
// record every child it queues: features (16 floats), mask words (stride 32),
// mass and instance index, up to max_items.  *count receives how many were
// recorded (children past max_items are not recorded).  Training data for the
// learned scorer.
extern "C" int nr_collect_children(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs,
                                   const int32_t *dsts, uint64_t capacity, const nr_options *opt,
                                   uint64_t max_items, float *feat, uint32_t *masks, double *mass, int32_t *inst,
                                   uint64_t *count, nr_result *res)
{
    if (!c || n <= 0 || !gs || !srcs || !dsts || !feat || !masks || !mass || !inst || !count || !res)
        return NR_ERR_INVALID;
    nr_options o;
    if (opt) o = *opt; else nr_options_default(&o);
    for (int i = 0; i < n; ++i) {
        memset(&res[i], 0, sizeof(nr_result));
        int rc = validate(&gs[i], srcs[i], dsts[i]);
        if (rc) return rc;
        if (gs[i].n_nodes > NR_SMALL_MAX_N) return NR_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(c->mu);
    drain(c);                          // finish batches in flight: slot 0 and the model are used here
    NR_CUDA_TRY(cudaSetDevice(c->device));
    if (o.order == NR_ORDER_LEARNED && !c->has_model) return NR_ERR_INVALID;
    if (o.branching != NR_BRANCH_PATH) return NR_ERR_UNSUPPORTED;    // features describe path children
    const bool exhaustive = !(o.target_width > 0) && o.order != NR_ORDER_MAXMASS && o.order != NR_ORDER_LEARNED;
    WarpRunCfg cfg = warp_cfg(&o, capacity, exhaustive);
    cfg.escalate = 0;                 // collect from whatever the warp engine reaches
    const int stride = 32;
    unsigned char *buf = nullptr;
    const size_t bytes = max_items * (NR_FEAT * sizeof(float) + stride * sizeof(uint32_t) + sizeof(double) +
                                      sizeof(int)) + 64;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) { cudaGetLastError(); return NR_ERR_NOMEM; }
    WarpDump d;
    d.count = reinterpret_cast<unsigned long long *>(buf);
    d.feat = reinterpret_cast<float *>(buf + 64);
    d.mask = reinterpret_cast<uint32_t *>(d.feat + max_items * NR_FEAT);
    d.mass = reinterpret_cast<double *>(d.mask + max_items * stride);
    d.inst = reinterpret_cast<int *>(d.mass + max_items);
    d.cap = max_items;
    d.stride = stride;
    cfg.dump = &d;
    int rc = NR_OK;
    unsigned long long got = 0;
    // the counter must be zero before the batch's own streams start
    if (cudaMemsetAsync(buf, 0, 64, c->stream) != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess)
        rc = NR_ERR_CUDA;
    std::vector<int> handover;
    if (!rc) rc = run_warp_batch(c, n, gs, srcs, dsts, cfg, res, &handover);
    if (!rc) {
        cudaStream_t s = c->stream;
        cudaMemcpyAsync(&got, d.count, sizeof(got), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        const unsigned long long k = std::min<unsigned long long>(got, max_items);
        if (k) {
            cudaMemcpyAsync(feat, d.feat, k * NR_FEAT * sizeof(float), cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(masks, d.mask, k * stride * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(mass, d.mass, k * sizeof(double), cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(inst, d.inst, k * sizeof(int), cudaMemcpyDeviceToHost, s);
        }
        if (cudaStreamSynchronize(s) != cudaSuccess) { cudaGetLastError(); rc = NR_ERR_CUDA; }
        *count = k;
    }
    cudaFree(buf);
    return rc;
}

extern "C" int nr_reliability_ctx(nr_context *c, const nr_graph *g, int src, int dst, uint64_t capacity,
                                  const nr_options *opt, nr_result *res)
{
    if (!c || !res) return NR_ERR_INVALID;
    memset(res, 0, sizeof(*res));
    int rc = validate(g, src, dst);
    if (rc) return rc;
    nr_options o;
    if (opt) o = *opt; else nr_options_default(&o);
    res->n_nodes = g->n_nodes;
    res->n_edges = g->n_edges;
    res->src = src;
    res->dst = dst;
    res->mask_words = std::max(1, (2 * g->n_edges + 31) / 32);
    std::lock_guard<std::mutex> lock(c->mu);
    drain(c);                          // finish batches in flight: slot 0 and the model are used here
    NR_CUDA_TRY(cudaSetDevice(c->device));
    if (o.branching != NR_BRANCH_PATH && o.branching != NR_BRANCH_FORK) return NR_ERR_INVALID;
    if (const int rb = branch_order_ok(c, o)) return rb;
    if (o.branch_order == NR_BORDER_LEARNED && g->n_nodes > NR_SMALL_MAX_N) return NR_ERR_UNSUPPORTED;
    if (o.branching == NR_BRANCH_FORK && o.order == NR_ORDER_LEARNED) return NR_ERR_UNSUPPORTED;
    if (g->n_nodes > NR_SMALL_MAX_N) return run_wide(c, g, src, dst, capacity, &o, res);
    if (o.target_width > 0 || o.order == NR_ORDER_MAXMASS || o.order == NR_ORDER_LEARNED) {
        // bucketed max-mass (or learned) order: one warp owns the instance (nr_warp.cuh)
        if (o.order == NR_ORDER_LEARNED && !c->has_model) return NR_ERR_INVALID;
        const WarpRunCfg cfg = warp_cfg(&o, capacity, false);
        std::vector<int> handover;
        int rc = run_warp_batch(c, 1, g, &src, &dst, cfg, res, &handover);
        if (rc) return rc;
        if (!handover.empty()) return NR_ERR_INTERNAL;
        return NR_OK;
    }
    // the wave engine's queue: the reference default capacity (common.h:33) when none is given
    return run_grid_small(c, g, src, dst, capacity ? capacity : (1u << 20), &o, res);
}

extern "C" int nr_reliability_kterminal(nr_context *c, const nr_graph *g, const int32_t *terminals, int n_terminals,
                                        uint64_t capacity, const nr_options *opt, nr_result *res)
{
    if (!c || !res || !terminals || n_terminals < 1) return NR_ERR_INVALID;
    memset(res, 0, sizeof(*res));
    const int src = terminals[0];
    for (int i = 0; i < n_terminals; ++i) {
        const int rc = validate(g, src, terminals[i]);
        if (rc) return rc;
    }
    nr_options o;
    if (opt) o = *opt; else nr_options_default(&o);
    if (o.order == NR_ORDER_LEARNED || o.branching != NR_BRANCH_PATH || o.branch_order != NR_BORDER_SRC)
        return NR_ERR_UNSUPPORTED;
    res->n_nodes = g->n_nodes;
    res->n_edges = g->n_edges;
    res->src = src;
    res->dst = terminals[n_terminals - 1];
    res->mask_words = std::max(1, (2 * g->n_edges + 31) / 32);
    std::lock_guard<std::mutex> lock(c->mu);
    drain(c);
    NR_CUDA_TRY(cudaSetDevice(c->device));
    // one terminal besides src is the two-terminal problem on the same engine (dst = that terminal)
    return run_wide(c, g, src, terminals[n_terminals - 1], capacity, &o, res, terminals, n_terminals);
}

// ---------------------------------------------------------------------------
// checkpoint / resume of a bucketed whole-GPU run
// file: "NRCKPT1" magic, run fingerprint, sizes, exact sums, counts, waves, then
// the live records (mask words, FP64 mass) one after another
// ---------------------------------------------------------------------------
namespace {
struct NrCkptHeader {
    char magic[8];
    uint64_t fp;
    int32_t n, E, src, dst, W4, pad;
    NrFix R, et, es, net;
    uint64_t nodes, leaves, dead, trunc, spilled, max_wave;
    int64_t waves;
    uint64_t live;
};
const char kCkptMagic[8] = {'N', 'R', 'C', 'K', 'P', 'T', '1', 0};
}  // namespace

extern "C" int nr_checkpoint_save(nr_context *c, const char *path)
{
    if (!c || !path) return NR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(c->mu);
    const NrCkptState &k = c->ckpt;
    if (!k.valid) return NR_ERR_INVALID;
    NR_CUDA_TRY(cudaSetDevice(c->device));
    unsigned long long top = 0;
    NR_CUDA_TRY(cudaMemcpy(&top, static_cast<unsigned char *>(c->sbuf) + k.off_top, sizeof(top),
                           cudaMemcpyDeviceToHost));
    const size_t used = (size_t)std::min<unsigned long long>(top, k.cap);
    const size_t rec = 16 * (size_t)k.W4;
    const unsigned char *qb = static_cast<const unsigned char *>(c->qbuf);
    std::vector<unsigned char> keys(used), masks(used * rec);
    std::vector<double> mass(used);
    if (used) {
        NR_CUDA_TRY(cudaMemcpy(keys.data(), qb + k.mask_bytes + k.mass_bytes, used, cudaMemcpyDeviceToHost));
        NR_CUDA_TRY(cudaMemcpy(masks.data(), qb, used * rec, cudaMemcpyDeviceToHost));
        NR_CUDA_TRY(cudaMemcpy(mass.data(), qb + k.mask_bytes, used * sizeof(double), cudaMemcpyDeviceToHost));
    }
    NrCkptHeader h;
    memset(&h, 0, sizeof(h));
    memcpy(h.magic, kCkptMagic, 8);
    h.fp = k.fp;
    h.n = k.n; h.E = k.E; h.src = k.src; h.dst = k.dst; h.W4 = k.W4;
    h.R = k.R; h.et = k.et; h.es = k.es; h.net = k.net;
    h.nodes = k.nodes; h.leaves = k.leaves; h.dead = k.dead; h.trunc = k.trunc; h.spilled = k.spilled;
    h.max_wave = k.max_wave;
    h.waves = k.waves;
    for (size_t i = 0; i < used; ++i) h.live += (keys[i] != NR_WIDE_FREE);
    FILE *f = fopen(path, "wb");
    if (!f) return NR_ERR_IO;
    bool ok = fwrite(&h, sizeof(h), 1, f) == 1;
    for (size_t i = 0; i < used && ok; ++i) {
        if (keys[i] == NR_WIDE_FREE) continue;
        ok = fwrite(masks.data() + i * rec, 1, rec, f) == rec && fwrite(&mass[i], sizeof(double), 1, f) == 1;
    }
    ok = (fclose(f) == 0) && ok;
    return ok ? NR_OK : NR_ERR_IO;
}

extern "C" int nr_checkpoint_resume(nr_context *c, const char *path, const nr_graph *g, int src, int dst,
                                    uint64_t capacity, const nr_options *opt, nr_result *res)
{
    if (!c || !path || !res) return NR_ERR_INVALID;
    memset(res, 0, sizeof(*res));
    int rc = validate(g, src, dst);
    if (rc) return rc;
    nr_options o;
    if (opt) o = *opt; else nr_options_default(&o);
    if (g->n_nodes <= NR_SMALL_MAX_N || o.bucket_shift < 0 || o.order == NR_ORDER_LEARNED) return NR_ERR_UNSUPPORTED;
    if (o.branching != NR_BRANCH_PATH && o.branching != NR_BRANCH_FORK) return NR_ERR_INVALID;
    FILE *f = fopen(path, "rb");
    if (!f) return NR_ERR_IO;
    NrCkptHeader h;
    NrResumeIn rin;
    bool ok = fread(&h, sizeof(h), 1, f) == 1 && memcmp(h.magic, kCkptMagic, 8) == 0;
    const int W4 = std::max(1, ((2 * g->n_edges + 31) / 32 + 3) / 4);
    ok = ok && h.fp == nr_run_fingerprint(g, src, dst, &o) && h.W4 == W4 && h.live < (1ull << 32);
    if (!ok) { fclose(f); return NR_ERR_INVALID; }
    const size_t rec = 16 * (size_t)W4;
    rin.masks.resize(h.live * rec);
    rin.mass.resize(h.live);
    for (uint64_t i = 0; i < h.live && ok; ++i)
        ok = fread(rin.masks.data() + i * rec, 1, rec, f) == rec && fread(&rin.mass[i], sizeof(double), 1, f) == 1;
    fclose(f);
    if (!ok) return NR_ERR_PARSE;
    rin.R = h.R; rin.et = h.et; rin.es = h.es; rin.net = h.net;
    rin.nodes = h.nodes; rin.leaves = h.leaves; rin.dead = h.dead; rin.trunc = h.trunc; rin.spilled = h.spilled;
    rin.max_wave = h.max_wave;
    rin.waves = h.waves;
    res->n_nodes = g->n_nodes; res->n_edges = g->n_edges; res->src = src; res->dst = dst;
    res->mask_words = std::max(1, (2 * g->n_edges + 31) / 32);
    std::lock_guard<std::mutex> lock(c->mu);
    drain(c);
    NR_CUDA_TRY(cudaSetDevice(c->device));
    return run_bucket_wide(c, g, src, dst, capacity ? capacity : (1u << 22), &o, res, &rin);
}

extern "C" int nr_reliability(const nr_graph *g, int src, int dst, uint64_t capacity, const nr_options *opt,
                              nr_result *res)
{
    if (!res) return NR_ERR_INVALID;
    memset(res, 0, sizeof(*res));
    int rc = validate(g, src, dst);
    if (rc) return rc;
    nr_context *c = nullptr;
    rc = nr_context_create(opt ? opt->device : 0, &c);
    if (rc) return rc;
    rc = nr_reliability_ctx(c, g, src, dst, capacity, opt, res);
    nr_context_destroy(c);
    return rc;
}
