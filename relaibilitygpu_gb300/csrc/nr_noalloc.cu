// nr_noalloc.cu -- nr_reliability_noalloc: one instance, no device allocation.
//
// Some callers cannot call cudaMalloc: a host application whose device
// memory is owned by its own allocator or memory pool, a plugin that may not
// grow the process footprint, or code running where allocation is forbidden
// or too slow to do per call.  This entry point solves one instance with the
// warp-per-instance engine (nr_warp.cuh) using only the file-scope static
// device array below for everything the solve needs on the device: the
// graph tables, the work counter, the per-instance output and the queue
// pages.  It calls no cudaMalloc, cudaFree or other allocating routine.
//
// Limits and behaviour:
//   * the array is NR_NOALLOC_SCRATCH_BYTES (4 MiB) on every GPU that loads
//     the library, held until the process exits;
//   * graphs must have n_nodes <= 32 and tables that fit in the array; larger
//     inputs are rejected with NR_ERR_UNSUPPORTED;
//   * the queue gets whatever the tables leave (at most 8192 pages of 32
//     subproblems); when it is full, child mass is spilled into ESP as the
//     reference does on queue overflow (workingPad/main.cu:245-252), so the
//     result stays a valid R <= true <= R + ESP bracket;
//   * the first call on a device looks up the array's device address with
//     cudaGetSymbolAddress (set-up, once per device, with that device
//     current); make that first call before any stream capture;
//   * every call reuses the same array, which keeps the previous call's
//     contents: the work counter is cleared at the start of each call, and
//     the kernel writes every other byte it reads before reading it;
//   * calls are serialised by a process-wide lock and each waits for its
//     kernel, but work that overlaps with a call on the GPU and touches the
//     array (another process cannot: it has its own copy) would race;
//   * it runs on cudaStreamPerThread and reports the in-kernel device time
//     (globaltimer) as ms, because timing events are created resources;
//   * one warp does the whole solve, so every run has a pop budget: max_nodes,
//     or NR_NOALLOC_DEFAULT_BUDGET (2^24 pops, enough for exhaustive K10) when it
//     is 0.  A run that reaches it stops with stop = 3 and a valid
//     R <= true <= R + ESP bracket (the mass still queued is part of ESP);
//   * the caller's current device is restored before the call returns.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <mutex>

#include "nr_internal.h"
#include "nr_warp.cuh"

const void *nr_warp_kernel_ptr_g8(int w4);
const void *nr_warp_kernel_ptr_g16(int w4);
const void *nr_warp_kernel_ptr_g32(int w4);
const void *nr_warp_fork_kernel_ptr_g8(int w4);
const void *nr_warp_fork_kernel_ptr_g16(int w4);
const void *nr_warp_fork_kernel_ptr_g32(int w4);

#define NR_NOALLOC_SCRATCH_BYTES (4u << 20)
#define NR_NOALLOC_MAX_DEVICES 64
#define NR_NOALLOC_BLOB_MAX (32u << 10)
#define NR_NOALLOC_DEFAULT_BUDGET (1ull << 24)

static __device__ __align__(256) unsigned char nr_noalloc_scratch[NR_NOALLOC_SCRATCH_BYTES];

namespace {

std::mutex g_noalloc_mu;
unsigned char *g_noalloc_addr[NR_NOALLOC_MAX_DEVICES];
unsigned char g_noalloc_blob[NR_NOALLOC_BLOB_MAX];   // host staging for the graph tables

size_t a16(size_t x) { return (x + 15) & ~size_t(15); }

// Puts the calling thread's current device back when the call returns.
struct DeviceRestore {
    int prev = -1;
    DeviceRestore() { if (cudaGetDevice(&prev) != cudaSuccess) { cudaGetLastError(); prev = -1; } }
    ~DeviceRestore() { if (prev >= 0) cudaSetDevice(prev); }
};
size_t a256(size_t x) { return (x + 255) & ~size_t(255); }

// Graph tables in the layout of NrSmallGraph (nr_internal.h), written into
// the fixed host buffer; returns the byte count or 0 if they do not fit.
size_t noalloc_tables(const nr_graph *g, int src, int dst, int G, NrSmallGraph *sg)
{
    const int n = g->n_nodes, E = g->n_edges;
    const int W = std::max(1, (2 * E + 31) / 32);
    sg->n = n; sg->e = E; sg->w4 = (W + 3) / 4; sg->src = src; sg->dst = dst; sg->n_in = g->n_arcs;
    sg->rows = 0; sg->off_root_rows = 0;
    size_t off = 0;
    sg->off_p = (int)off; off = a16(off + sizeof(double) * std::max(E, 1));
    sg->off_eid = (int)off; off = a16(off + sizeof(uint16_t) * G * G);
    sg->off_start = (int)off; off = a16(off + sizeof(int) * (n + 1));
    sg->off_list = (int)off; off = a16(off + sizeof(uint32_t) * std::max(g->n_arcs, 1));
    sg->blob_bytes = (int)off;
    sg->blob_off = 0;
    sg->struct_off = 0;
    if (off > NR_NOALLOC_BLOB_MAX) return 0;
    unsigned char *b = g_noalloc_blob;
    memset(b, 0, off);
    double *p = reinterpret_cast<double *>(b + sg->off_p);
    uint16_t *eid = reinterpret_cast<uint16_t *>(b + sg->off_eid);
    int *start = reinterpret_cast<int *>(b + sg->off_start);
    uint32_t *list = reinterpret_cast<uint32_t *>(b + sg->off_list);
    for (int e = 0; e < E; ++e) p[e] = g->edge_p[e];
    for (int i = 0; i < G * G; ++i) eid[i] = 0xffff;
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
            if (eid[u * G + v] == 0xffff) eid[u * G + v] = (uint16_t)e;
        }
    return off;
}

}  // namespace

extern "C" int nr_reliability_noalloc(const nr_graph *g, int src, int dst, const nr_options *opt, nr_result *res)
{
    if (!g || !res) return NR_ERR_INVALID;
    memset(res, 0, sizeof(*res));
    if (g->n_nodes <= 0 || !g->row_ptr || src < 0 || dst < 0 || src >= g->n_nodes || dst >= g->n_nodes)
        return NR_ERR_INVALID;
    if (g->n_arcs < 0 || g->n_edges < 0 || (g->n_arcs > 0 && (!g->col_idx || !g->edge_id)) ||
        (g->n_edges > 0 && !g->edge_p) || g->row_ptr[0] != 0 || g->row_ptr[g->n_nodes] != g->n_arcs)
        return NR_ERR_INVALID;
    for (int u = 0; u < g->n_nodes; ++u)
        if (g->row_ptr[u + 1] < g->row_ptr[u]) return NR_ERR_INVALID;
    for (int j = 0; j < g->n_arcs; ++j)
        if (g->col_idx[j] < 0 || g->col_idx[j] >= g->n_nodes || g->edge_id[j] < 0 || g->edge_id[j] >= g->n_edges)
            return NR_ERR_INVALID;
    for (int e = 0; e < g->n_edges; ++e)        // a NaN p would feed NaN masses into the exact sums
        if (std::isnan(g->edge_p[e])) return NR_ERR_INVALID;
    if (g->n_nodes > NR_SMALL_MAX_N) return NR_ERR_UNSUPPORTED;
    nr_options o;
    if (opt) o = *opt; else nr_options_default(&o);
    const int dev = o.device;
    if (dev < 0 || dev >= NR_NOALLOC_MAX_DEVICES) return NR_ERR_INVALID;

    if (o.branching != NR_BRANCH_PATH && o.branching != NR_BRANCH_FORK) return NR_ERR_INVALID;
    if (o.branch_order < NR_BORDER_SRC || o.branch_order > NR_BORDER_LEARNED) return NR_ERR_INVALID;
    if (o.branch_order == NR_BORDER_LEARNED) return NR_ERR_UNSUPPORTED;   // no scorer here

    std::lock_guard<std::mutex> lock(g_noalloc_mu);
    DeviceRestore restore;
    if (cudaSetDevice(dev) != cudaSuccess) { cudaGetLastError(); return NR_ERR_CUDA; }
    if (!g_noalloc_addr[dev]) {     // set-up, once per device, with the device current
        void *p = nullptr;
        if (cudaGetSymbolAddress(&p, nr_noalloc_scratch) != cudaSuccess || !p) {
            cudaGetLastError();
            return NR_ERR_CUDA;
        }
        g_noalloc_addr[dev] = static_cast<unsigned char *>(p);
    }
    unsigned char *base = g_noalloc_addr[dev];

    const int G = g->n_nodes <= 8 ? 8 : g->n_nodes <= 16 ? 16 : 32;
    NrSmallGraph sg;
    const size_t blob = noalloc_tables(g, src, dst, G, &sg);
    if (!blob || sg.w4 > NR_MAX_W4) return NR_ERR_UNSUPPORTED;
    const bool fork = (o.branching == NR_BRANCH_FORK);
    const void *kfn = fork ? (G == 8 ? nr_warp_fork_kernel_ptr_g8(sg.w4) : G == 16 ? nr_warp_fork_kernel_ptr_g16(sg.w4)
                                                                              : nr_warp_fork_kernel_ptr_g32(sg.w4))
                           : (G == 8 ? nr_warp_kernel_ptr_g8(sg.w4) : G == 16 ? nr_warp_kernel_ptr_g16(sg.w4)
                                                                         : nr_warp_kernel_ptr_g32(sg.w4));
    if (!kfn) return NR_ERR_UNSUPPORTED;

    // array layout: tables | descriptor | id | counter | output | page masks | page masses
    size_t off = a256(blob);
    const size_t off_desc = off; off = a16(off + sizeof(NrSmallGraph));
    const size_t off_id = off; off = a16(off + sizeof(int));
    const size_t off_cnt = off; off = a16(off + sizeof(int));
    const size_t off_out = off; off = a256(off + sizeof(NrWarpOut));
    const size_t item = 16 * (size_t)sg.w4 + sizeof(double);
    const size_t room = NR_NOALLOC_SCRATCH_BYTES > off ? NR_NOALLOC_SCRATCH_BYTES - off : 0;
    int pages = (int)std::min<size_t>(8192, room / (NR_PAGE * item + 16));
    if (pages < 4) return NR_ERR_UNSUPPORTED;
    const size_t off_mask = off;
    const size_t off_mass = a256(off_mask + (size_t)pages * NR_PAGE * 16 * sg.w4);
    if (off_mass + (size_t)pages * NR_PAGE * sizeof(double) > NR_NOALLOC_SCRATCH_BYTES) return NR_ERR_UNSUPPORTED;

    const bool exhaustive = !(o.target_width > 0) && o.order != NR_ORDER_MAXMASS && o.order != NR_ORDER_LEARNED;
    NrWarpParams P;
    P.blob = base;
    P.inst = reinterpret_cast<const NrSmallGraph *>(base + off_desc);
    P.inst_id = reinterpret_cast<const int *>(base + off_id);
    P.n_inst = 1;
    P.next_inst = reinterpret_cast<int *>(base + off_cnt);
    P.slab_mask = reinterpret_cast<uint4 *>(base + off_mask);
    P.slab_mass = reinterpret_cast<double *>(base + off_mass);
    P.slab_rows = nullptr;            // rows are rebuilt from the masks (no room budgeted for them)
    P.pages = pages;
    P.escalate = 0;
    P.eps = o.truncation_eps > 0 ? o.truncation_eps : 0.0;
    P.target = o.target_width > 0 ? o.target_width : 0.0;
    P.target_fix = nr_fix_of(P.target);
    // Exhaustive runs take one page at a time (depth first: the queue stays small); the others
    // run the wave schedule of their order.  Both stop at the budget with their queue intact.
    const unsigned long long budget = o.max_nodes ? o.max_nodes : NR_NOALLOC_DEFAULT_BUDGET;
    if (exhaustive) {
        P.wave_mode = 0; P.shift = -1; P.n_buckets = 32; P.max_nodes = budget;
    } else {
        P.wave_mode = 1; P.shift = o.bucket_shift;
        P.n_buckets = std::min(1024, ((o.n_buckets > 0 ? o.n_buckets : 256) + 31) / 32 * 32);
        P.max_nodes = budget;
    }
    P.out = reinterpret_cast<NrWarpOut *>(base + off_out);
    P.learned = 0;
    P.fork = (o.branching == NR_BRANCH_FORK);
    P.dump_feat = nullptr; P.dump_mask = nullptr; P.dump_mass = nullptr; P.dump_inst = nullptr;
    P.dump_count = nullptr; P.dump_cap = 0; P.dump_stride = 0; P.inst_base = 0;
    P.step_cap = 0;
    P.border = o.branch_order;
    P.handover_pages = 0;
    P.row_words = 0;

    const size_t smem = nr_warp_shm_bytes(32 / G, sg.w4, P.n_buckets, pages);
    cudaStream_t s = cudaStreamPerThread;
    const int zero = 0;
    NrWarpOut out;
    cudaError_t e = nr_smem_limit(dev, kfn, smem);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base, g_noalloc_blob, blob, cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + off_desc, &sg, sizeof(sg), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(base + off_id, &zero, sizeof(int), cudaMemcpyHostToDevice, s);
    if (e == cudaSuccess) e = cudaMemsetAsync(base + off_cnt, 0, sizeof(int), s);   // clear the work counter
    void *args[] = {&P};
    if (e == cudaSuccess) e = cudaLaunchKernel(kfn, dim3(1), dim3(32), args, smem, s);
    if (e == cudaSuccess) e = cudaMemcpyAsync(&out, base + off_out, sizeof(out), cudaMemcpyDeviceToHost, s);
    if (e == cudaSuccess) e = cudaStreamSynchronize(s);
    if (e != cudaSuccess) { cudaGetLastError(); return NR_ERR_CUDA; }

    res->n_nodes = g->n_nodes; res->n_edges = g->n_edges; res->src = src; res->dst = dst;
    res->mask_words = std::max(1, (2 * g->n_edges + 31) / 32);
    NrFix esp = out.et;
    nr_fix_add_host(esp, out.es);
    nr_fix_add_host(esp, out.q);
    res->R = nr_fix_to_double_host(out.R);
    res->esp = nr_fix_to_double_host(esp);
    res->R_plus_esp = res->R + res->esp;
    res->trunc_bound = res->R > 0 ? res->esp / res->R : res->esp;
    res->nodes = out.nodes; res->leaves = out.leaves; res->dead_ends = out.dead; res->truncated = out.trunc;
    res->spilled = out.spilled; res->paths = out.leaves + out.spilled; res->queued = out.queued;
    res->iterations = out.waves;
    res->max_queue_items = out.max_wave;
    res->item_bytes = (int)item;
    res->max_queue_mb = (double)out.max_wave * item / (1024.0 * 1024.0);
    res->ms = out.t_ns / 1e6;
    res->time_to_bound_ms = out.t_ns / 1e6;
    res->engine = NR_ENGINE_WARP;
    res->grid_blocks = 1;
    res->block_threads = 32;
    res->capacity = (uint64_t)pages * NR_PAGE;
    res->h2d_bytes = blob + sizeof(sg) + sizeof(int);
    res->d2h_bytes = sizeof(out);
    // With no hand-over (escalate = 0) a page-mode stop (status 2) can only be the budget: the
    // queued mass is still counted in ESP, so the bracket is valid, as for a wave-mode budget stop.
    res->stop = (out.status == 2) ? 3 : out.status;
    if (out.status < 0 || out.status > 3) return NR_ERR_INTERNAL;
    return NR_OK;
}
