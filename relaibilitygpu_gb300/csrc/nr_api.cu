// nr_api.cu -- host side of the C ABI declared in include/nr.h: options, contexts, the
// single-instance engines (whole-GPU waves for n <= 32, the wide engines), checkpoints,
// K-terminal runs.  The batch runtime is nr_batch.cu, the loader and result block nr_io.cu.
//
// Replaces the reference driver (workingPad/main.cu:795-1072) with calls that return status codes.

#include "nr_host.h"

thread_local char g_err[256];
thread_local char g_internal[128];      // which device-side check failed, when one says

// keep the failing call and its line for nr_status_string
void nr_last_cuda_error(cudaError_t e, const char *file, int line, const char *what)
{
    const char *base = strrchr(file, '/');
    snprintf(g_err, sizeof(g_err), "%s (%s:%d %.120s)", cudaGetErrorString(e), base ? base + 1 : file, line, what);
}


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
int ensure(void **buf, size_t *have, size_t need)
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
int validate_shape(const nr_graph *g, int src, int dst)
{
    if (!g || g->n_nodes <= 0 || g->n_edges < 0 || g->n_arcs < 0 || !g->row_ptr) return NR_ERR_INVALID;
    if (g->n_arcs > 0 && (!g->col_idx || !g->edge_id)) return NR_ERR_INVALID;
    if (g->n_edges > 0 && !g->edge_p) return NR_ERR_INVALID;
    if (src < 0 || dst < 0 || src >= g->n_nodes || dst >= g->n_nodes) return NR_ERR_INVALID;
    return NR_OK;
}

int validate_probabilities(const nr_graph *g)
{
    for (int e = 0; e < g->n_edges; ++e)
        if (std::isnan(g->edge_p[e])) return NR_ERR_INVALID;
    return NR_OK;
}

// The CSR arrays: row offsets, heads and edge ids in range.
int validate_structure(const nr_graph *g)
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
bool same_structure_arrays(const nr_graph *a, const nr_graph *b)
{
    return a->n_nodes == b->n_nodes && a->n_arcs == b->n_arcs && a->n_edges == b->n_edges &&
           a->row_ptr == b->row_ptr && a->col_idx == b->col_idx && a->edge_id == b->edge_id;
}

int validate(const nr_graph *g, int src, int dst)
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
int rows_mode_of(const nr_graph *g)
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
size_t small_inst_layout(const nr_graph *g, int src, int dst, NrSmallGraph *sg)
{
    const int n = g->n_nodes, E = g->n_edges;
    const int W = std::max(1, (2 * E + 31) / 32);
    sg->n = n; sg->e = E; sg->w4 = (W + 3) / 4; sg->src = src; sg->dst = dst;
    sg->n_in = g->n_arcs;
    sg->rows = 0;
    sg->off_root_rows = 0;
    size_t off = 0;
    sg->off_p = (int)off; off = align16(off + sizeof(double) * std::max(E, 1));
    return off;
}

// Structural part: offsets of the edge-id table and in-arc lists from base `at`.
size_t small_struct_layout(const nr_graph *g, NrSmallGraph *sg, size_t at)
{
    const int n = g->n_nodes, G = group_width_of(n);
    size_t off = at;
    sg->off_eid = (int)off; off = align16(off + sizeof(uint16_t) * G * G);
    sg->off_start = (int)off; off = align16(off + sizeof(int) * (n + 1));
    sg->off_list = (int)off; off = align16(off + sizeof(uint32_t) * std::max(g->n_arcs, 1));
    sg->off_root_rows = (int)off; off = align16(off + sizeof(uint32_t) * 32);
    return off - at;
}

// Copies p; false if one of them is NaN.
bool small_fill_inst(const nr_graph *g, const NrSmallGraph *sg, unsigned char *b)
{
    const int E = g->n_edges;
    double *p = reinterpret_cast<double *>(b + sg->off_p);
    memcpy(p, g->edge_p, sizeof(double) * E);
    int nan = 0;
    for (int e = 0; e < E; ++e) nan |= p[e] != p[e];     // no early exit: the loop vectorizes
    return nan == 0;
}

void small_fill_struct(const nr_graph *g, const NrSmallGraph *sg, unsigned char *b)
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
    // the rows of a lane kernel's root when no edge is certainly down: n <= 16, 16-bit rows two
    // to a word; n <= 32, one 32-bit row a word
    uint32_t *rr = reinterpret_cast<uint32_t *>(b + sg->off_root_rows);
    for (int k = 0; k < 32; ++k) rr[k] = 0u;
    for (int u = 0; u < n && n <= 32; ++u)
        for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; ++j) {
            const int v = g->col_idx[j];
            if (n <= 16) rr[v >> 1] |= 1u << (u + ((v & 1) << 4));
            else rr[v] |= 1u << u;
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
bool same_topology(const nr_graph *a, const nr_graph *b)
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
        nr_last_cuda_error(e, __FILE__, __LINE__, "context set-up");
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
        if (sl.hv_dev) cudaFree(sl.hv_dev);
        if (sl.hv_host) cudaFreeHost(sl.hv_host);
        for (int k = 0; k < NR_HV_STREAMS; ++k) {
            if (sl.hv_side[k]) cudaStreamDestroy(sl.hv_side[k]);
            if (sl.hv_join[k]) cudaEventDestroy(sl.hv_join[k]);
        }
        if (sl.hv_fork) cudaEventDestroy(sl.hv_fork);
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

int run_grid_small(nr_context *c, const nr_graph *g, int src, int dst, uint64_t cap,
                          const nr_options *o, nr_result *r)
{
    c->ckpt.valid = false;                 // the arena is about to be reused
    NrSmallGraph sg;
    std::vector<unsigned char> blob;
    build_small_blob(g, src, dst, &sg, &blob);
    const int G = group_width(g->n_nodes);
    const int W4 = sg.w4;
    if (W4 > NR_MAX_W4) return NR_ERR_UNSUPPORTED;
    // one lane per subproblem (nr_grid_lane.cuh) on undirected simple graphs with path branching,
    // unless the lane groups are asked for: graphs of <= 16 nodes
    // (16-bit rows), or of <= 32 nodes (32-bit rows)
    const int rb = g->n_nodes <= NR_LANE_MAX_N ? 16 : 32;
    const bool lane = o->branching != NR_BRANCH_FORK && o->small_kernel != NR_SMALL_GROUP &&
                      W4 <= (rb == 16 ? NR_LANE_MAX_W4 : NR_LANE32_MAX_W4) && rows_mode_of(g) == 1 &&
                      cap <= 0x7fffffffull;
    const void *kfn = lane ? nr_grid_lane_kernel_ptr(W4, rb) : grid_kernel(G, W4, o->branching == NR_BRANCH_FORK);
    if (!kfn) return NR_ERR_UNSUPPORTED;

    const int block = NR_BLOCK_THREADS;
    const int warps = block / 32;
    const size_t smem = lane ? nr_grid_lane_shm_bytes(sg.blob_bytes, warps, rb)
                             : (size_t)sg.blob_bytes + (size_t)warps * (32 / G) * 4 * W4 * sizeof(uint32_t);
    NR_CUDA_TRY(nr_smem_limit(c->device, kfn, smem));
    int bps = 0;
    NR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kfn, block, smem));
    if (bps < 1) return NR_ERR_UNSUPPORTED;
    if (o->blocks_per_sm > 0 && o->blocks_per_sm < bps) bps = o->blocks_per_sm;
    const int grid = bps * c->sms;

    const size_t row_bytes = lane ? (rb == 16 ? 4 * (size_t)NR_LANE_ROW_WORDS : 128) : 0;   // rows in the records
    const size_t item_bytes = (size_t)W4 * 16 + sizeof(double) + row_bytes;
    const size_t mask_bytes = align16((size_t)cap * W4 * 16);
    const size_t mass_bytes = align16((size_t)cap * sizeof(double));
    const size_t rows_bytes = align16((size_t)cap * row_bytes);
    const size_t qneed = 2 * (mask_bytes + mass_bytes + rows_bytes);
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
    P.rows[0] = lane ? reinterpret_cast<uint4 *>(qb + 2 * (mask_bytes + mass_bytes)) : nullptr;
    P.rows[1] = lane ? reinterpret_cast<uint4 *>(qb + 2 * (mask_bytes + mass_bytes) + rows_bytes) : nullptr;
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
    // the root's not-down rows (lane kernel): node v's in-neighbours over edges with p > 0, two
    // 16-bit rows a word, or one 32-bit row a word
    uint32_t root_rows[32] = {0};
    if (lane) {
        for (int u = 0; u < g->n_nodes; ++u)
            for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; ++j)
                if (g->edge_p[g->edge_id[j]] > 0.0) {
                    const int v = g->col_idx[j];
                    if (rb == 16) root_rows[v >> 1] |= 1u << (u + ((v & 1) << 4));
                    else root_rows[v] |= 1u << u;
                }
        NR_CUDA_TRY(cudaMemcpyAsync(P.rows[0], root_rows, row_bytes, cudaMemcpyHostToDevice, s));
    }

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
    r->kernel = lane ? NR_KERNEL_LANE : 0;
    r->grid_blocks = grid;
    r->block_threads = block;
    r->capacity = cap;
    r->h2d_bytes = blob.size() + sizeof(one_u) + 16 * W4 + sizeof(one) + row_bytes;
    r->d2h_bytes = sizeof(unsigned long long) * wc.size() + sizeof(NrPartial) * grid + sizeof(int);
    if (status & NR_DEV_ERR_TIMEOUT) return NR_ERR_TIMEOUT;
    if (status) return NR_ERR_INTERNAL;
    return NR_OK;
}

// ---------------------------------------------------------------------------
// whole-GPU engine for 33..16384 nodes (nr_wide.cuh)
// ---------------------------------------------------------------------------
// The bitset search's conditions: at most NR_WIDE_BITS_MAX_N nodes, no self-loop, no two arcs
// with the same tail and head, no edge id on more than two arcs.
static bool wide_bits_ok(const nr_graph *g)
{
    const int n = g->n_nodes, E = g->n_edges;
    if (n > NR_WIDE_BITS_MAX_N) return false;
    std::vector<unsigned char> uses(std::max(E, 1), 0);
    uint32_t seen[NR_WIDE_BITS_MAX_N / 32];
    for (int u = 0; u < n; ++u) {
        memset(seen, 0, sizeof(seen));
        for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; ++j) {
            const int w = g->col_idx[j], e = g->edge_id[j];
            if (w == u || ((seen[w >> 5] >> (w & 31)) & 1u) || ++uses[e] > 2) return false;
            seen[w >> 5] |= 1u << (w & 31);
        }
    }
    return true;
}

static void build_wide_blob(const nr_graph *g, int src, int dst, NrWideGraph *wg, std::vector<unsigned char> *blob,
                            const int32_t *terms = nullptr, int nt = 0, bool fork = false)
{
    const int n = g->n_nodes, E = g->n_edges;
    // the bitset search serves two-terminal path branching (the fork's up-only search and the
    // K-terminal visit order walk the out-arcs)
    wg->bitset = (!fork && nt == 0 && wide_bits_ok(g)) ? 1 : 0;
    const int W = std::max(1, (2 * E + 31) / 32);
    wg->n = n; wg->e = E; wg->w4 = (W + 3) / 4; wg->src = src; wg->dst = dst; wg->n_arcs = g->n_arcs;
    wg->nwd = (n + 31) / 32;
    size_t off = 0;
    wg->off_p = (int)off; off = align16(off + sizeof(double) * std::max(E, 1));
    wg->off_row = (int)off; off = align16(off + sizeof(int) * (n + 1));
    wg->off_arc = (int)off; off = align16(off + sizeof(uint32_t) * std::max(g->n_arcs, 1));
    wg->off_kmask = (int)off; off = align16(off + sizeof(uint32_t) * wg->nwd);
    wg->off_rows = wg->off_ehead = 0;
    if (wg->bitset) {
        wg->off_rows = (int)off; off = align16(off + sizeof(uint32_t) * (size_t)n * wg->nwd);
        wg->off_ehead = (int)off; off = align16(off + sizeof(uint32_t) * std::max(E, 1));
    }
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
    int *row = reinterpret_cast<int *>(blob->data() + wg->off_row);
    uint32_t *arc = reinterpret_cast<uint32_t *>(blob->data() + wg->off_arc);
    for (int e = 0; e < E; ++e) p[e] = g->edge_p[e];
    if (wg->bitset) {
        // in-arcs (eid << 14 | tail) grouped by head, out-neighbour rows, heads of each edge
        uint32_t *rows = reinterpret_cast<uint32_t *>(blob->data() + wg->off_rows);
        uint32_t *eh = reinterpret_cast<uint32_t *>(blob->data() + wg->off_ehead);
        for (int e = 0; e < E; ++e) eh[e] = 0xffffffffu;
        std::vector<int> fill(n + 1, 0);
        for (int j = 0; j < g->n_arcs; ++j) fill[g->col_idx[j] + 1]++;
        for (int w = 0; w < n; ++w) fill[w + 1] += fill[w];
        for (int w = 0; w <= n; ++w) row[w] = fill[w];
        for (int u = 0; u < n; ++u)
            for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; ++j) {
                const int w = g->col_idx[j], e = g->edge_id[j];
                arc[fill[w]++] = ((uint32_t)e << NR_WIDE_HEAD_BITS) | (uint32_t)u;
                rows[(size_t)u * wg->nwd + (w >> 5)] |= 1u << (w & 31);
                eh[e] = ((eh[e] & 0xffffu) == 0xffffu) ? (0xffff0000u | (uint32_t)w) : ((eh[e] & 0xffffu) | ((uint32_t)w << 16));
            }
    } else {
        for (int u = 0; u <= n; ++u) row[u] = g->row_ptr[u];
        for (int j = 0; j < g->n_arcs; ++j)
            arc[j] = ((uint32_t)g->edge_id[j] << NR_WIDE_HEAD_BITS) | (uint32_t)g->col_idx[j];
    }
    wg->tables_global = off > NR_WIDE_STAGE_MAX;
}

int smem_optin(nr_context *c)
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
    if (o->branch_order == NR_BORDER_LEARNED) return NR_ERR_UNSUPPORTED;   // the bucketed queue only
    c->ckpt.valid = false;                 // the arena is about to be reused
    if (g->n_nodes > NR_WIDE_MAX_N || g->n_edges > 65535) return NR_ERR_UNSUPPORTED;
    NrWideGraph wg;
    std::vector<unsigned char> blob;
    build_wide_blob(g, src, dst, &wg, &blob, terms, nt, o->branching == NR_BRANCH_FORK);
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

// Several graphs above 32 nodes in breadth-first waves (path branching), side by side: the
// instances of one mask width share a cooperative launch, each on its own group of blocks
// (nr_grid_wide_multi_kernel), as many per launch as the grid and the device memory hold.  Every
// instance follows run_grid_wide's schedule, so its results are run_grid_wide's.
int run_grid_wide_multi(nr_context *c, const std::vector<int> &idx, const nr_graph *gs, const int32_t *srcs,
                        const int32_t *dsts, uint64_t cap, const nr_options *o, nr_result *res)
{
    if (o->branch_order == NR_BORDER_LEARNED) return NR_ERR_UNSUPPORTED;   // the bucketed queue only
    c->ckpt.valid = false;                 // the arena is about to be reused
    struct Inst { int i; NrWideGraph wg; std::vector<unsigned char> blob; };
    std::vector<Inst> all;
    all.reserve(idx.size());
    for (int i : idx) {
        if (gs[i].n_nodes > NR_WIDE_MAX_N || gs[i].n_edges > 65535) return NR_ERR_UNSUPPORTED;
        Inst in;
        in.i = i;
        build_wide_blob(&gs[i], srcs[i], dsts[i], &in.wg, &in.blob);
        all.push_back(std::move(in));
    }
    std::stable_sort(all.begin(), all.end(), [](const Inst &a, const Inst &b) {
        return std::min(a.wg.w4, NR_WIDE_MAX_W4 + 1) < std::min(b.wg.w4, NR_WIDE_MAX_W4 + 1);
    });
    const long long timeout_ns = (long long)((o->timeout_ms > 0 ? o->timeout_ms : 60000.0) * 1e6);
    size_t at = 0;
    while (at < all.size()) {
        // a run of instances with one compiled mask width (wider masks share the runtime width)
        const int key = std::min(all[at].wg.w4, NR_WIDE_MAX_W4 + 1);
        size_t end = at;
        while (end < all.size() && std::min(all[end].wg.w4, NR_WIDE_MAX_W4 + 1) == key) ++end;
        const void *kfn = nr_grid_wide_multi_kernel_ptr(key);
        if (!kfn) return NR_ERR_UNSUPPORTED;
        int block = NR_WIDE_BLOCK;
        size_t smem = 0;
        for (size_t k = at; k < end; ++k) block = std::min(block, wide_block(c, all[k].wg));
        if (!block) return NR_ERR_UNSUPPORTED;
        for (size_t k = at; k < end; ++k) smem = std::max(smem, nr_wide_block_shm(all[k].wg, block / 32));
        NR_CUDA_TRY(nr_smem_limit(c->device, kfn, smem));
        int bps = 0;
        NR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kfn, block, smem));
        if (bps < 1) return NR_ERR_UNSUPPORTED;
        if (o->blocks_per_sm > 0 && o->blocks_per_sm < bps) bps = o->blocks_per_sm;
        const int grid_max = bps * c->sms;
        int maxw4 = 1, max_waves = 2;
        for (size_t k = at; k < end; ++k) {
            maxw4 = std::max(maxw4, all[k].wg.w4);
            max_waves = std::max(max_waves, all[k].wg.e + 2);
        }
        // instances per launch: one block each at least, and their wave buffers in device memory
        const size_t per_inst = 2 * (align16((size_t)cap * maxw4 * 16) + align16((size_t)cap * sizeof(double)));
        size_t free_b = 0, total_b = 0;
        NR_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
        const size_t budget = std::max(per_inst, (free_b + c->qbytes) / 2);
        const size_t m_mem = std::max<size_t>(1, budget / per_inst);
        for (size_t c0 = at; c0 < end;) {
            // at least a block per SM for each instance: an instance's widest waves need the warps
            // (on the uneven batch's 6x6 grids, 152 blocks each ran 1.35x faster than 6 each)
            const int m = (int)std::min<size_t>({end - c0, (size_t)std::max(1, grid_max / c->sms), m_mem});
            const int bpi = grid_max / m, grid = bpi * m;
            const size_t mask_b = align16((size_t)cap * maxw4 * 16), mass_b = align16((size_t)cap * sizeof(double));
            int rc = ensure(&c->qbuf, &c->qbytes, (size_t)m * 2 * (mask_b + mass_b));
            if (rc) return rc;
            // control buffer: tables, graphs, offsets, roots, counters, barriers, partials, shares, stops
            size_t off = 0;
            std::vector<long long> boff(m);
            for (int k = 0; k < m; ++k) { boff[k] = (long long)off; off = align16(off + all[c0 + k].blob.size()); }
            const size_t off_g = off; off = align16(off + sizeof(NrWideGraph) * m);
            const size_t off_bo = off; off = align16(off + sizeof(long long) * m);
            const size_t off_root = off; off = align16(off + (size_t)16 * maxw4 * m);
            const size_t off_wc = off; off = align16(off + sizeof(unsigned long long) * (max_waves + 1) * m);
            const size_t off_bar = off; off = align16(off + 4 * sizeof(unsigned) * m);
            const size_t off_part = off; off = align16(off + sizeof(NrPartial) * grid);
            const size_t off_wpart = off; off = align16(off + sizeof(NrWideShare) * 2 * grid);
            const size_t off_stop = off; off = align16(off + 2 * sizeof(int) * m);
            rc = ensure(&c->sbuf, &c->sbytes, off);
            if (rc) return rc;
            std::vector<unsigned char> up(off_wc, 0);
            std::vector<NrWideGraph> gv(m);
            std::vector<uint32_t> roots((size_t)4 * maxw4 * m, 0);
            for (int k = 0; k < m; ++k) {
                const Inst &in = all[c0 + k];
                memcpy(up.data() + boff[k], in.blob.data(), in.blob.size());
                gv[k] = in.wg;
                nr_initial_mask(&gs[in.i], roots.data() + (size_t)4 * maxw4 * k, 4 * in.wg.w4);
            }
            memcpy(up.data() + off_g, gv.data(), sizeof(NrWideGraph) * m);
            memcpy(up.data() + off_bo, boff.data(), sizeof(long long) * m);
            memcpy(up.data() + off_root, roots.data(), (size_t)16 * maxw4 * m);
            unsigned char *sb = static_cast<unsigned char *>(c->sbuf);
            unsigned char *qb = static_cast<unsigned char *>(c->qbuf);
            NrGridWideMultiParams P;
            P.g = reinterpret_cast<const NrWideGraph *>(sb + off_g);
            P.blob = sb;
            P.blob_off = reinterpret_cast<const long long *>(sb + off_bo);
            P.root = reinterpret_cast<const uint4 *>(sb + off_root);
            P.mask = reinterpret_cast<uint4 *>(qb);
            P.mass = reinterpret_cast<double *>(qb + (size_t)m * 2 * mask_b);
            P.mask_half = mask_b / 16;
            P.mass_half = mass_b / sizeof(double);
            P.capacity = cap;
            P.wave_count = reinterpret_cast<unsigned long long *>(sb + off_wc);
            P.max_waves = max_waves;
            P.bar = reinterpret_cast<unsigned *>(sb + off_bar);
            P.partials = reinterpret_cast<NrPartial *>(sb + off_part);
            P.wpart = reinterpret_cast<NrWideShare *>(sb + off_wpart);
            P.stop_wave = reinterpret_cast<int *>(sb + off_stop);
            P.m = m;
            P.bpi = bpi;
            P.eps = o->truncation_eps > 0 ? o->truncation_eps : 0.0;
            P.timeout_ns = timeout_ns;
            P.target_on = o->target_width > 0 ? 1 : 0;
            P.target_fix = nr_fix_of(o->target_width > 0 ? o->target_width : 0.0);
            P.max_nodes = o->max_nodes;
            P.border = o->branch_order;
            cudaStream_t s = c->stream;
            NR_CUDA_TRY(cudaMemcpyAsync(sb, up.data(), up.size(), cudaMemcpyHostToDevice, s));
            NR_CUDA_TRY(cudaMemsetAsync(sb + off_wc, 0, off - off_wc, s));
            void *args[] = {&P};
            NR_CUDA_TRY(cudaEventRecord(c->ev0, s));
            NR_CUDA_TRY(cudaLaunchCooperativeKernel(kfn, dim3(grid), dim3(block), args, smem, s));
            NR_CUDA_TRY(cudaEventRecord(c->ev1, s));
            std::vector<unsigned long long> wc((size_t)(max_waves + 1) * m);
            std::vector<NrPartial> parts(grid);
            std::vector<unsigned> bars((size_t)4 * m);
            std::vector<int> stops((size_t)2 * m);
            NR_CUDA_TRY(cudaMemcpyAsync(wc.data(), P.wave_count, sizeof(unsigned long long) * wc.size(),
                                        cudaMemcpyDeviceToHost, s));
            NR_CUDA_TRY(cudaMemcpyAsync(parts.data(), P.partials, sizeof(NrPartial) * grid, cudaMemcpyDeviceToHost, s));
            NR_CUDA_TRY(cudaMemcpyAsync(bars.data(), P.bar, sizeof(unsigned) * bars.size(), cudaMemcpyDeviceToHost, s));
            NR_CUDA_TRY(cudaMemcpyAsync(stops.data(), P.stop_wave, sizeof(int) * stops.size(), cudaMemcpyDeviceToHost, s));
            NR_CUDA_TRY(cudaStreamSynchronize(s));
            float ms = 0.f;
            NR_CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
            int status_all = 0;
            for (int k = 0; k < m; ++k) {
                const Inst &in = all[c0 + k];
                nr_result *r = &res[in.i];
                const int status = (int)bars[(size_t)4 * k + 2];
                status_all |= status;
                NrFix R = nr_fix_zero(), esp = nr_fix_zero();
                unsigned long long nodes = 0, leaves = 0, dead = 0, trunc = 0, spilled = 0;
                for (int b = k * bpi; b < (k + 1) * bpi; ++b) {
                    const NrPartial &pp = parts[b];
                    nr_fix_add(R, pp.R);
                    nr_fix_add(esp, pp.et);
                    nr_fix_add(esp, pp.es);
                    nr_fix_add(esp, pp.q);      // still queued at a target stop
                    nodes += pp.nodes; leaves += pp.leaves; dead += pp.dead; trunc += pp.truncated;
                    spilled += pp.spilled;
                }
                const unsigned long long *w = wc.data() + (size_t)(max_waves + 1) * k;
                const int stop_wave = stops[2 * k];
                int waves = 0;
                unsigned long long maxw = 0, queued = 0;
                const int last = stop_wave >= 0 ? stop_wave : max_waves + 1;
                for (int q = 0; q <= max_waves && q < last; ++q) {
                    const unsigned long long nn = std::min<unsigned long long>(w[q], cap);
                    if (!nn) break;
                    waves++;
                    maxw = std::max(maxw, nn);
                }
                if (stop_wave >= 0) queued = std::min<unsigned long long>(w[stop_wave], cap);
                const size_t item_bytes = (size_t)in.wg.w4 * 16 + sizeof(double);
                r->R = nr_fix_to_double_host(R);
                r->esp = nr_fix_to_double_host(esp);
                r->R_plus_esp = r->R + r->esp;
                r->trunc_bound = r->R > 0 ? r->esp / r->R : r->esp;
                r->nodes = nodes; r->leaves = leaves; r->dead_ends = dead; r->truncated = trunc; r->spilled = spilled;
                r->paths = leaves + spilled;
                r->queued = queued;
                r->stop = stop_wave >= 0 ? stops[2 * k + 1] : 0;
                r->iterations = waves;
                r->max_queue_items = maxw;
                r->item_bytes = (int)item_bytes;
                r->max_queue_mb = (double)maxw * item_bytes / (1024.0 * 1024.0);
                r->ms = ms;
                if (stop_wave >= 0 && stops[2 * k + 1] == 1) r->time_to_bound_ms = ms;
                r->engine = NR_ENGINE_GRID;
                r->grid_blocks = bpi;
                r->block_threads = block;
                r->capacity = cap;
                r->h2d_bytes = in.blob.size() + sizeof(NrWideGraph) + sizeof(long long) + 16 * maxw4;
                r->d2h_bytes = sizeof(unsigned long long) * (max_waves + 1) + sizeof(NrPartial) * bpi +
                               6 * sizeof(int);
            }
            if (status_all & NR_DEV_ERR_TIMEOUT) return NR_ERR_TIMEOUT;
            if (status_all) return NR_ERR_INTERNAL;
            c0 += m;
        }
        at = end;
    }
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

// Every edge id on exactly the two arcs u -> v and v -> u, no self-loop, no ordered pair twice.
static bool undirected_simple(const nr_graph *g)
{
    const int n = g->n_nodes, E = g->n_edges;
    if (g->n_arcs != 2 * E) return false;
    std::vector<int> cnt(std::max(E, 1), 0), tail(std::max(E, 1), -1), head(std::max(E, 1), -1);
    std::vector<std::pair<int, int>> pairs;
    pairs.reserve(g->n_arcs);
    for (int u = 0; u < n; ++u)
        for (int j = g->row_ptr[u]; j < g->row_ptr[u + 1]; ++j) {
            const int v = g->col_idx[j], e = g->edge_id[j];
            if (v == u || e < 0 || e >= E) return false;
            if (cnt[e]++ == 0) { tail[e] = u; head[e] = v; }
            else if (tail[e] != v || head[e] != u) return false;   // the second arc is v -> u
            pairs.push_back({u, v});
        }
    for (int e = 0; e < E; ++e)
        if (cnt[e] != 2) return false;
    std::sort(pairs.begin(), pairs.end());
    return std::adjacent_find(pairs.begin(), pairs.end()) == pairs.end();
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
    build_wide_blob(g, src, dst, &wg, &blob, terms, nt, o->branching == NR_BRANCH_FORK);
    const int W4 = wg.w4;
    // the learned branch order: the scorer's kernel, its weights and scratch (two-terminal path
    // branching)
    const bool learn = o->branch_order == NR_BORDER_LEARNED;
    if (learn && (!c->has_model || nt > 0 || o->branching != NR_BRANCH_PATH)) return NR_ERR_UNSUPPORTED;
    // one lane per subproblem: undirected simple graphs of <= 250 nodes with the bit-set tables,
    // two-terminal path branching, the src-side-first branch order (small_kernel = group keeps a
    // warp per subproblem)
    const bool lanes = !learn && wg.bitset && nt == 0 && o->branching == NR_BRANCH_PATH &&
                       o->branch_order == NR_BORDER_SRC && o->small_kernel != NR_SMALL_GROUP &&
                       wg.n <= NR_WIDE_LANES_MAX_N && W4 >= 1 && W4 <= NR_WIDE_MAX_W4 && undirected_simple(g);
    const void *kfn = learn ? nr_bucket_wide_learn_kernel_ptr(W4)
                            : lanes ? nr_bucket_wide_lanes_kernel_ptr(W4) : nr_bucket_wide_kernel_ptr(W4);
    if (!kfn) return NR_ERR_UNSUPPORTED;
    const size_t learn_warp = learn ? (size_t)NR_WIDE_LEARN_WORDS * 4 : lanes ? nr_wide_lane_shm(wg.n, W4) : 0;
    int block = 0;
    for (int w = NR_WIDE_BLOCK / 32; w >= 1 && !block; --w)
        if (nr_wide_block_shm(wg, w) + w * learn_warp <= (size_t)smem_optin(c)) block = 32 * w;
    if (!block) return NR_ERR_UNSUPPORTED;
    const size_t smem = nr_wide_block_shm(wg, block / 32) + (block / 32) * learn_warp;
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
    P.mlp = c->mlp;                       // used by the learned instantiation only
    P.target_on = o->target_width > 0 ? 1 : 0;
    P.target_fix = nr_fix_of(o->target_width > 0 ? o->target_width : 0.0);
    P.max_nodes = o->max_nodes;
    P.wpart = reinterpret_cast<NrWideShare *>(sb + off_wpart);
    P.stop_info = reinterpret_cast<int *>(sb + off_info);
    P.stats = reinterpret_cast<unsigned long long *>(sb + off_stats);
    P.resume = rin ? 1 : 0;
    // one lane a record from waves of NR_WIDE_LANE_MIN_PER_WARP records a warp up
    P.lane_min_wave = (unsigned long long)NR_WIDE_LANE_MIN_PER_WARP * grid * (block / 32);
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
    r->kernel = lanes ? NR_KERNEL_LANE : 0;
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
int run_wide(nr_context *c, const nr_graph *g, int src, int dst, uint64_t capacity, const nr_options *o,
                    nr_result *r, const int32_t *terms, int nt)
{
    if (o->order == NR_ORDER_LEARNED) return NR_ERR_UNSUPPORTED;
    const bool buckets = o->bucket_shift >= 0 &&
                         (o->order == NR_ORDER_MAXMASS || (o->order == NR_ORDER_AUTO && o->target_width > 0));
    if (buckets) return run_bucket_wide(c, g, src, dst, capacity ? capacity : (1u << 22), o, r, nullptr, terms, nt);
    return run_grid_wide(c, g, src, dst, capacity ? capacity : (1u << 20), o, r, terms, nt);
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
    // graphs above 32 nodes take the learned branch order in the bucketed whole-GPU queue only
    if (o.branch_order == NR_BORDER_LEARNED && g->n_nodes > NR_SMALL_MAX_N &&
        !(o.bucket_shift >= 0 && (o.order == NR_ORDER_MAXMASS || (o.order == NR_ORDER_AUTO && o.target_width > 0))))
        return NR_ERR_UNSUPPORTED;
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

