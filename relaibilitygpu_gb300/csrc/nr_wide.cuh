// nr_wide.cuh -- whole-GPU engine for graphs with 33..16384 nodes.
//
// One warp per subproblem.  Node sets are bitmasks of ceil(n/32) words in
// the warp's shared memory.  Each BFS level compacts the frontier into a
// list, the lanes walk the out-arcs of its nodes (CSR, as listed in the file)
// and mark new nodes with atomicOr.  The parent of a node is taken with
// atomicMin on (u << 16 | edge), i.e. the smallest frontier node with a
// not-down arc to it -- the same deterministic rule as the small engines and
// the oracle, where the reference's multi-lane BFS races on parent[]
// (workingPad/device_code.cuh:165-170).  There is no path-length cap (the
// reference stops at 32 nodes, workingPad/main.cu:152).  Children are
// emitted in hop order with the lanes owning mask words, so every child
// record is written with coalesced stores.
//
// Two schedules share that step (nr_wide_step):
//  * nr_grid_wide_kernel -- breadth-first waves in ping-pong buffers, as the
//    reference's host loop (main.cu:963-1008), with the grid barrier, wave
//    counters and block partials of nr_grid.cuh;
//  * nr_bucket_wide_kernel -- the bucketed max-mass queue: records live in
//    one HBM arena with a bucket byte each (2^shift buckets per factor of two
//    in mass); every wave takes the whole highest non-empty bucket (a scan of
//    the bucket bytes gathers its slots) and children are appended to the
//    arena.  Slots freed by earlier waves are reclaimed by an in-place
//    compaction once they are a large part of the used arena.
//
// A target width stops either schedule before the first wave at which
// ESP + queued mass <= target (the oracle's wave schedule): at the end of a
// wave every block writes its exact share of that width (its ESP so far plus
// the mass it queued minus the mass it popped) to one of two alternating
// slots, and after the grid barrier every block adds all shares and takes the
// same decision.  The shares also carry node counts, for a node budget.
#pragma once

#include "nr_expand.cuh"
#include "nr_mlp.cuh"

#define NR_WIDE_MAX_N 16384     // arcs carry a 14-bit head; parents pack (node << 16 | edge)
#define NR_WIDE_MAX_W4 16       // widest mask with a compiled width; wider masks run the
                                // runtime-width instantiation (W4 = 0): masks up to 65535 edges
#define NR_WIDE_HEAD_BITS 14
#define NR_WIDE_STAGE_MAX (64u << 10)   // graph tables above this are read from global memory
#define NR_WIDE_BLOCK 128
#define NR_WIDE_MAX_NB 255      // bucket schedule: bucket ids fit a byte
#define NR_WIDE_FREE 0xffu      // bucket byte of a free arena slot

// Graph tables of one wide instance: p[E] (double), row_ptr[n+1] (int),
// arcs[n_arcs] (u32 = eid << 14 | head).  Offsets from the blob start, 16-byte aligned.
// Tables up to NR_WIDE_STAGE_MAX are staged into every block's shared memory; larger ones (the
// reference's 6301-node directed fixture: 440 KB) are read from global memory (L2).
// Bitset tables (bitset = 1; two-terminal path branching on graphs of <= NR_WIDE_BITS_MAX_N nodes
// without self-loops or parallel arcs): row/arc then hold the IN-arcs (u32 = eid << 14 | tail),
// rows[n][nwd] each node's out-neighbour bitmask, ehead[E] the heads of an edge's arcs (low and
// high 16 bits; 0xffff: none).
struct NrWideGraph {
    int n, e, w4, src, dst, n_arcs, nwd;
    int off_p, off_row, off_arc, blob_bytes;
    int nk;                     // K-terminal: terminals other than src (0: two-terminal, dst)
    int off_kmask;              // K-terminal: bitmask of the terminals, nwd words
    int tables_global;          // 1: the tables stay in global memory
    int bitset;                 // 1: the bitset search (nr_wide_bfs_bits) and its tables
    int off_rows, off_ehead;
};
#define NR_WIDE_BITS_MAX_N 256  // bitset search: nwd <= 8 words, levels fit a byte

// A block's share of the stop test, written at the end of each wave.
struct NrWideShare {
    NrFix width;                // ESP so far + (mass queued - mass popped)
    unsigned long long nodes;   // subproblems popped so far
    unsigned long long pad;
};

struct NrGridWideParams {
    NrWideGraph g;
    const unsigned char *blob;
    uint4 *mask[2];
    double *mass[2];
    unsigned long long capacity;
    unsigned long long *wave_count;
    int max_waves;
    unsigned *bar_count;
    unsigned *bar_gen;
    int *status;
    NrPartial *partials;
    double eps;
    long long timeout_ns;
    int target_on;                  // stop at ESP + queued <= target_fix
    NrFix target_fix;
    unsigned long long max_nodes;   // stop once this many subproblems were popped (0 = no budget)
    NrWideShare *wpart;             // [2][gridDim.x] per-block shares, alternating slots
    int *stop_wave;                 // [0] waves run before a stop (or -1), [1] stop reason
    int fork;                       // 1: fork branching on the most reliable path edge
    int border;                     // NR_BORDER_*: the order a path's UNKNOWN edges are branched in
};

struct NrBucketWideParams {
    NrWideGraph g;
    const unsigned char *blob;
    uint4 *mask;                    // arena [capacity][w4]
    double *mass;                   // arena [capacity]
    unsigned char *key;             // arena [capacity]: bucket, or NR_WIDE_FREE
    unsigned *list;                 // [capacity]: slots of the running wave; compaction scratch
    unsigned long long capacity;
    unsigned long long *top;        // arena slots handed out (slots >= capacity were spilled)
    unsigned long long *bcount;     // [nb] records per bucket
    unsigned long long *wave_len;   // [2] gathered slots, alternating
    unsigned long long *ccount;     // [2][gridDim.x] compaction counts
    int shift, nb, max_waves;
    unsigned *bar_count;
    unsigned *bar_gen;
    int *status;
    NrPartial *partials;
    double eps;
    long long timeout_ns;
    int target_on;
    NrFix target_fix;
    unsigned long long max_nodes;
    NrWideShare *wpart;
    int *stop_info;                 // [0] waves run, [1] stop reason (0 empty, 1 target, 3 budget), [2] compactions
    unsigned long long *stats;      // [0] widest wave, [1] records queued at the end
    int fork;                       // 1: fork branching on the most reliable path edge
    int border;                     // NR_BORDER_*: the order a path's UNKNOWN edges are branched in
    NrMlpDev mlp;                   // the learned branch order's scorer (the LEARN instantiation)
    // resume from a checkpoint: the arena holds its queue and block 0's first lane starts from
    // its sums and counts (the stop test before the first wave sees them through the shares)
    int resume;
    NrFix init_R, init_et, init_es, init_net;
    unsigned long long init_nodes, init_leaves, init_dead, init_trunc, init_spilled;
    unsigned long long lane_min_wave;   // LANES: the smallest wave run one lane a record
};

// per-warp shared memory: mask words, a working copy of them (runtime-width children),
// frontier / next / visited bitmasks (nwd words each, at least 32), packed parents, frontier
// list, path hops, K-terminal visit order.  Rounded to 16 bytes: each warp's region starts with
// the mask, which is written with 16-byte stores.
__host__ __device__ inline int nr_wide_nwd32(int n) { return (((n + 31) / 32 + 31) / 32) * 32; }
__host__ __device__ inline size_t nr_wide_warp_shm(int n, int w4)
{
    return ((((size_t)8 * w4 + 3 * (size_t)nr_wide_nwd32(n) + 4 * (size_t)n) * 4) + 15) & ~(size_t)15;
}

// shared memory of a block of `warps` warps: staged tables (unless read from global) + scratch
__host__ __device__ inline size_t nr_wide_block_shm(const NrWideGraph &g, int warps)
{
    return (g.tables_global ? 0 : (size_t)g.blob_bytes) + (size_t)warps * nr_wide_warp_shm(g.n, g.w4);
}

// Where a step's children go.
struct NrWideOut {
    uint4 *mask;
    double *mass;
    unsigned char *key;              // bucket schedule: bucket byte of each record, else nullptr
    unsigned long long *count;       // slots handed out so far; slots >= cap spill
    unsigned long long cap;
    int shift, nb;
    unsigned *hist;                  // bucket schedule: this block's new records per bucket (shared memory)
};

// Accumulators of a warp (its lane 0 updates them; they live in the block's shared memory).
struct NrWideAcc {
    NrFix R, et, es;
    NrFix net;                       // mass queued minus mass popped
    unsigned long long nodes, leaves, dead, trunc, spilled;
};

struct NrWideView {
    const double *p;                 // q = 1 - p is computed (__dsub_rn: the host's rounding)
    const int *row;
    const uint32_t *arc;
    const uint32_t *rows, *ehead;    // bitset tables (g.bitset)
    const uint32_t *kmask;           // K-terminal terminals (nullptr: two-terminal)
    uint32_t *m, *wk, *F, *NF, *VIS, *par, *list, *hops, *order;
};

// tables: the staged copy in shared memory, or the blob in global memory (g.tables_global)
__device__ __forceinline__ NrWideView nr_wide_view(unsigned char *smem, const unsigned char *blob,
                                                   const NrWideGraph &g)
{
    const int NW = 4 * g.w4, NWD = nr_wide_nwd32(g.n);
    const unsigned char *tb = g.tables_global ? blob : smem;
    NrWideView v;
    v.p = reinterpret_cast<const double *>(tb + g.off_p);
    v.row = reinterpret_cast<const int *>(tb + g.off_row);
    v.arc = reinterpret_cast<const uint32_t *>(tb + g.off_arc);
    v.rows = g.bitset ? reinterpret_cast<const uint32_t *>(tb + g.off_rows) : nullptr;
    v.ehead = g.bitset ? reinterpret_cast<const uint32_t *>(tb + g.off_ehead) : nullptr;
    const int warp = threadIdx.x >> 5;
    uint32_t *ws = reinterpret_cast<uint32_t *>(smem + (g.tables_global ? 0 : g.blob_bytes) +
                                                (size_t)warp * nr_wide_warp_shm(g.n, g.w4));
    v.m = ws;                        // [NW] mask words of the current subproblem
    v.wk = v.m + NW;                 // [NW] working copy (runtime-width children)
    v.F = v.wk + NW;                 // [NWD] frontier
    v.NF = v.F + NWD;                // [NWD] next frontier
    v.VIS = v.NF + NWD;              // [NWD] visited
    v.par = v.VIS + NWD;             // [n] (parent << 16) | edge
    v.list = v.par + g.n;            // [n] frontier nodes
    v.hops = v.list + g.n;           // [n] path edges, dst side first
    v.order = v.hops + g.n;          // [n] K-terminal: visit order of the search
    v.kmask = g.nk ? reinterpret_cast<const uint32_t *>(tb + g.off_kmask) : nullptr;
    return v;
}

// Load a record's mask (w4 16-byte blocks) into the warp's shared copy.
__device__ __forceinline__ void nr_wide_load_mask(uint32_t *m, const uint4 *src, int w4)
{
    for (int k = threadIdx.x & 31; k < w4; k += 32) reinterpret_cast<uint4 *>(m)[k] = __ldcg(src + k);
}

// Two-terminal BFS of the warp from src over the arcs whose edge is not down
// (up_only: up), with the parent rule above; true if dst is reached.  The
// frontier is a node list: the lanes take its nodes, walk their arcs two at a
// time (independent loads), and the first discoverer of a node (the atomicOr
// that set its bit) appends it to the next list, so no level compacts a
// bitmask; the parent is still the atomicMin over every discovering arc of
// the level.  v.list and v.order hold the two lists, v.F[0] the next count.
__device__ __forceinline__ bool nr_wide_bfs_tt(const NrWideGraph &g, const NrWideView &v, bool up_only)
{
    const int lane = threadIdx.x & 31;
    const int n = g.n, nwd = g.nwd, src = g.src, dst = g.dst;
    const uint32_t *m = v.m;
    uint32_t *NF = v.NF, *VIS = v.VIS, *par = v.par, *cnt = v.F;
    uint32_t *cur = v.list, *nxt = v.order;
    const uint32_t sel = up_only ? 3u : 1u;      // usable: state & sel == 01 (01 or 11; up_only: 01)
    constexpr uint32_t HM = (1u << NR_WIDE_HEAD_BITS) - 1u;
    for (int i = lane; i < nwd; i += 32) {
        VIS[i] = 0u;
        NF[i] = 0u;
    }
    for (int i = lane; i < n; i += 32) par[i] = 0xffffffffu;
    __syncwarp();
    if (lane == 0) {
        VIS[src >> 5] = 1u << (src & 31);
        cur[0] = (uint32_t)src;
    }
    int f = 1;
    bool found = (src == dst);
    for (int level = 0; !found && f > 0 && level < n; ++level) {
        if (lane == 0) cnt[0] = 0u;
        __syncwarp();
        for (int i = lane; i < f; i += 32) {
            const uint32_t u = cur[i];
            const int j1 = v.row[u + 1];
            int j = v.row[u];
            auto visit = [&](uint32_t w, uint32_t e) {
                const uint32_t bit = 1u << (w & 31);
                const uint32_t old = atomicOr(&NF[w >> 5], bit);
                atomicMin(&par[w], (u << 16) | e);
                if (!(old & bit)) nxt[atomicAdd(cnt, 1u)] = w;
            };
            for (; j + 2 <= j1; j += 2) {
                const uint32_t a0 = v.arc[j], a1 = v.arc[j + 1];
                const uint32_t w0 = a0 & HM, e0 = a0 >> NR_WIDE_HEAD_BITS;
                const uint32_t w1 = a1 & HM, e1 = a1 >> NR_WIDE_HEAD_BITS;
                const uint32_t s0 = (m[e0 >> 4] >> ((e0 & 15) << 1)) & sel;
                const uint32_t s1 = (m[e1 >> 4] >> ((e1 & 15) << 1)) & sel;
                const uint32_t q0 = (VIS[w0 >> 5] >> (w0 & 31)) & 1u;
                const uint32_t q1 = (VIS[w1 >> 5] >> (w1 & 31)) & 1u;
                if (s0 == 1u && !q0) visit(w0, e0);
                if (s1 == 1u && !q1) visit(w1, e1);
            }
            if (j < j1) {
                const uint32_t a0 = v.arc[j];
                const uint32_t w0 = a0 & HM, e0 = a0 >> NR_WIDE_HEAD_BITS;
                if (((m[e0 >> 4] >> ((e0 & 15) << 1)) & sel) == 1u && !((VIS[w0 >> 5] >> (w0 & 31)) & 1u))
                    visit(w0, e0);
            }
        }
        __syncwarp();
        for (int i = lane; i < nwd; i += 32) {
            const uint32_t nf = NF[i];
            if (nf) {
                VIS[i] |= nf;
                NF[i] = 0u;
            }
        }
        __syncwarp();
        f = (int)cnt[0];
        found = (VIS[dst >> 5] >> (dst & 31)) & 1u;
        uint32_t *t = cur;
        cur = nxt;
        nxt = t;
        __syncwarp();
    }
    return found;
}

// Two-terminal BFS on node bitsets (g.bitset).  The next level is the union of
// the frontier's out-neighbour rows less the visited set; a new node that is
// the head of a down arc (the set H, from the mask's 00 states) stays only if
// one of its in-arcs from the frontier has a not-down edge, so the levels are
// those of the search over not-down arcs.  Word k of a union is OR-ed by the
// lanes k, k + nwp, ... (nwp: nwd rounded up to a power of two) and combined
// by shuffles; no atomics on the search's state.  Levels go to lvl[] (the
// bytes of v.par), the frontier lists to v.list / v.order in ascending node
// order; the parents follow on the path only (nr_wide_path_bits).
__device__ __forceinline__ bool nr_wide_bfs_bits(const NrWideGraph &g, const NrWideView &v)
{
    constexpr uint32_t HM = (1u << NR_WIDE_HEAD_BITS) - 1u;
    const int lane = threadIdx.x & 31;
    const int n = g.n, nwd = g.nwd, src = g.src, dst = g.dst, E = g.e;
    const uint32_t *m = v.m;
    uint32_t *F = v.F, *VIS = v.VIS, *H = v.NF;
    uint8_t *lvl = reinterpret_cast<uint8_t *>(v.par);
    uint32_t *cur = v.list, *nxt = v.order;
    if (lane < nwd) { H[lane] = 0u; VIS[lane] = 0u; F[lane] = 0u; }
    __syncwarp();
    // H: heads of the arcs of the down edges (00 states; mask bits past edge E-1 are padding)
    for (int k = lane; k < 4 * g.w4 && 16 * k < E; k += 32) {
        const uint32_t w = m[k];
        for (uint32_t dn = ~w & ~(w >> 1) & 0x55555555u; dn; dn &= dn - 1) {
            const int e = 16 * k + ((__ffs(dn) - 1) >> 1);
            if (e >= E) break;
            const uint32_t hh = v.ehead[e];
            atomicOr(&H[(hh & 0xffffu) >> 5], 1u << (hh & 31u));
            if ((hh >> 16) != 0xffffu) atomicOr(&H[(hh >> 16) >> 5], 1u << ((hh >> 16) & 31u));
        }
    }
    __syncwarp();
    if (lane == 0) {
        VIS[src >> 5] = 1u << (src & 31);
        F[src >> 5] = 1u << (src & 31);
        cur[0] = (uint32_t)src;
        lvl[src] = 0;
    }
    __syncwarp();
    const int nwp = nwd <= 1 ? 1 : nwd <= 2 ? 2 : nwd <= 4 ? 4 : 8;
    const int k = lane & (nwp - 1), part = lane / nwp, parts = 32 / nwp;
    int f = 1;
    bool found = (src == dst);
    for (int level = 0; !found && f > 0 && level < n; ++level) {
        uint32_t acc = 0u;
        if (k < nwd)
            for (int i = part; i < f; i += parts) acc |= v.rows[cur[i] * nwd + k];
        for (int off = nwp; off < 32; off <<= 1) acc |= __shfl_xor_sync(NR_FULL, acc, off);
        uint32_t nw = 0u;
        if (lane < nwd) {
            nw = acc & ~VIS[lane];
            for (uint32_t dn = nw & H[lane]; dn; dn &= dn - 1) {
                const int b = __ffs(dn) - 1;
                const int w = 32 * lane + b;
                bool ok = false;
                for (int j = v.row[w]; j < v.row[w + 1] && !ok; ++j) {
                    const uint32_t a = v.arc[j];
                    const uint32_t u = a & HM, e = a >> NR_WIDE_HEAD_BITS;
                    ok = ((F[u >> 5] >> (u & 31)) & 1u) && ((m[e >> 4] >> ((e & 15) << 1)) & 1u);
                }
                if (!ok) nw &= ~(1u << b);
            }
        }
        __syncwarp();                               // the checks above read F
        if (lane < nwd) {
            VIS[lane] |= nw;
            F[lane] = nw;
        }
        const int c = __popc(nw);                   // 0 on lanes >= nwd
        int pre = c;
#pragma unroll
        for (int off = 1; off < 8; off <<= 1) {
            const int t = __shfl_up_sync(NR_FULL, pre, off);
            if (lane >= off) pre += t;
        }
        f = __shfl_sync(NR_FULL, pre, 7);
        if (lane < nwd) {
            int o = pre - c;
            for (uint32_t b = nw; b; b &= b - 1) {
                const int w = 32 * lane + __ffs(b) - 1;
                nxt[o++] = (uint32_t)w;
                lvl[w] = (uint8_t)(level + 1);
            }
        }
        found = (__shfl_sync(NR_FULL, nw, dst >> 5) >> (dst & 31)) & 1u;
        uint32_t *t = cur;
        cur = nxt;
        nxt = t;
        __syncwarp();
    }
    return found;
}

// Path of a bitset search, dst back to src: the parent of x is the smallest
// (u << 16 | edge) over x's in-arcs from level lvl[x] - 1 whose edge is not
// down -- the parent rule of the other searches, evaluated on the path only.
// Writes hops[0..L) dst side first and returns L on every lane.
__device__ __forceinline__ int nr_wide_path_bits(const NrWideGraph &g, const NrWideView &v, uint32_t *hops)
{
    constexpr uint32_t HM = (1u << NR_WIDE_HEAD_BITS) - 1u;
    const int lane = threadIdx.x & 31;
    const uint8_t *lvl = reinterpret_cast<const uint8_t *>(v.par);
    const uint32_t *VIS = v.VIS, *m = v.m;
    int x = g.dst, h = 0;
    while (x != g.src && h < g.n) {
        const int want = (int)lvl[x] - 1;
        uint32_t best = 0xffffffffu;
        for (int j = v.row[x] + lane; j < v.row[x + 1]; j += 32) {
            const uint32_t a = v.arc[j];
            const uint32_t u = a & HM, e = a >> NR_WIDE_HEAD_BITS;
            if (((VIS[u >> 5] >> (u & 31)) & 1u) && (int)lvl[u] == want && ((m[e >> 4] >> ((e & 15) << 1)) & 1u))
                best = min(best, (u << 16) | e);
        }
        best = __reduce_min_sync(NR_FULL, best);
        if (best == 0xffffffffu) break;             // not reached: x came from level lvl[x] - 1
        if (lane == 0) hops[h] = best & 0xffffu;
        ++h;
        x = (int)(best >> 16);
    }
    __syncwarp();
    return h;
}

// BFS of the warp from src over the arcs whose edge is not down (up_only:
// up), with the parent rule above; true if dst is reached.  All 32 lanes call it.
// K-terminal (n_order given) keeps the bitmask frontier, whose compaction
// yields the visit order; two-terminal searches take nr_wide_bfs_tt.
__device__ __forceinline__ bool nr_wide_bfs(const NrWideGraph &g, const NrWideView &v, bool up_only,
                                            int *n_order = nullptr)
{
    if (n_order == nullptr) return nr_wide_bfs_tt(g, v, up_only);
    const int lane = threadIdx.x & 31;
    const int n = g.n, nwd = g.nwd, src = g.src, dst = g.dst;
    const uint32_t *m = v.m;
    uint32_t *F = v.F, *NF = v.NF, *VIS = v.VIS, *par = v.par, *list = v.list;
    // usable state: 01 or 11 (bit 0 set), or exactly 01
    const uint32_t want = up_only ? 1u : 1u, sel = up_only ? 3u : 1u;
    for (int i = lane; i < nwd; i += 32) {
        VIS[i] = 0u;
        F[i] = 0u;
    }
    for (int i = lane; i < n; i += 32) par[i] = 0xffffffffu;
    __syncwarp();
    if (lane == 0) {
        VIS[src >> 5] = 1u << (src & 31);
        F[src >> 5] = 1u << (src & 31);
    }
    __syncwarp();
    // K-terminal (n_order given): search until every terminal is reached, recording the
    // visit order (src, then each level in ascending node order) in v.order
    const bool kmode = n_order != nullptr;
    int no = 0;
    bool found = kmode ? (g.nk == 0) : (src == dst);
    while (!found) {
        // compact the frontier into list[] (and, K-terminal, append it to the visit order),
        // 32 bitmask words at a time
        int total = 0;
        for (int c = 0; c < nwd; c += 32) {
            const uint32_t fw = (c + lane < nwd) ? F[c + lane] : 0u;
            const int cnt = __popc(fw);
            int pre = cnt;
            for (int off = 1; off < 32; off <<= 1) {
                const int t = __shfl_up_sync(NR_FULL, pre, off);
                if (lane >= off) pre += t;
            }
            int o = total + pre - cnt;
            for (uint32_t b = fw; b; b &= b - 1) list[o++] = (uint32_t)((c + lane) * 32 + __ffs(b) - 1);
            if (kmode) {
                int oo = no + total + pre - cnt;
                for (uint32_t b = fw; b; b &= b - 1) v.order[oo++] = (uint32_t)((c + lane) * 32 + __ffs(b) - 1);
            }
            total += __shfl_sync(NR_FULL, pre, 31);
        }
        if (total == 0) break;
        if (kmode) no += total;
        for (int i = lane; i < nwd; i += 32) NF[i] = 0u;
        __syncwarp();
        for (int i = lane; i < total; i += 32) {
            const uint32_t u = list[i];
            for (int j = v.row[u]; j < v.row[u + 1]; ++j) {
                const uint32_t a = v.arc[j];
                const uint32_t w = a & ((1u << NR_WIDE_HEAD_BITS) - 1u), e = a >> NR_WIDE_HEAD_BITS;
                if (((m[e >> 4] >> ((e & 15) << 1)) & sel) == want && !((VIS[w >> 5] >> (w & 31)) & 1u)) {
                    atomicOr(&NF[w >> 5], 1u << (w & 31));
                    atomicMin(&par[w], (u << 16) | e);
                }
            }
        }
        __syncwarp();
        bool any = false;
        for (int i = lane; i < nwd; i += 32) {
            const uint32_t nf = NF[i];
            VIS[i] |= nf;
            F[i] = nf;
            any = any || nf != 0u;
        }
        __syncwarp();
        if (kmode) {
            bool all = true;
            for (int i = lane; i < nwd; i += 32) all = all && ((VIS[i] & v.kmask[i]) == v.kmask[i]);
            found = __all_sync(NR_FULL, all);
        } else {
            found = (VIS[dst >> 5] >> (dst & 31)) & 1u;
        }
        if (!__any_sync(NR_FULL, any)) break;
    }
    if (kmode && found) {
        // the last level searched: the new frontier, appended in ascending node order
        for (int c = 0; c < nwd; c += 32) {
            const uint32_t fw = (c + lane < nwd) ? F[c + lane] : 0u;
            const int cnt = __popc(fw);
            int pre = cnt;
            for (int off = 1; off < 32; off <<= 1) {
                const int t = __shfl_up_sync(NR_FULL, pre, off);
                if (lane >= off) pre += t;
            }
            int oo = no + pre - cnt;
            for (uint32_t b = fw; b; b &= b - 1) v.order[oo++] = (uint32_t)((c + lane) * 32 + __ffs(b) - 1);
            no += __shfl_sync(NR_FULL, pre, 31);
        }
        __syncwarp();
    }
    if (kmode) *n_order = no;
    return found;
}

// Write one child record (mask = m with edge e's state bits cleared by `clear`)
// at the next slot of O and count it; lanes own mask words (w4: the mask's 16-byte blocks).
__device__ __forceinline__ void nr_wide_emit(const NrWideOut &O, NrWideAcc &A, const uint32_t *m, int w4,
                                             unsigned long long slot, int e, uint32_t clear, double cm)
{
    const int lane = threadIdx.x & 31;
    const int wi = e >> 4;
    if (slot < O.cap) {
        uint32_t *dstw = reinterpret_cast<uint32_t *>(O.mask + slot * w4);
        for (int i = lane; i < 4 * w4; i += 32) __stcg(dstw + i, (i == wi) ? (m[i] & ~clear) : m[i]);
        if (lane == 0) {
            __stcg(O.mass + slot, cm);
            nr_fix_add_mass(A.net, cm);
            if (O.key) {
                const int b = nr_bucket(cm, O.shift, O.nb);
                __stcg(O.key + slot, (unsigned char)b);
                atomicAdd(&O.hist[b], 1u);
            }
        }
    } else if (lane == 0) {                                 // queue full (main.cu:245-252)
        A.spilled++;
        nr_fix_add_mass(A.es, cm);
    }
}

// Pop of one subproblem whose mask words are in v.m: count it, truncate it
// below eps, else BFS, and on a path emit the branches and the all-up leaf --
// or, with fork branching (main.cu:303-430 with :550-565), put the whole mass
// in R when a path of up edges exists, else fork on the optimistic path's
// UNKNOWN edge with the largest p (ties: nearest dst): down child, then up.
// All 32 lanes call it; the accumulators live on lane 0.
// Branch order of a path held dst side first in hops[0..L) (the children are made from
// hops[L-1] down to hops[0]): rewrite hops so that walk visits the UNKNOWN edges dst side
// first, or by p (ascending / descending, stable in path order: the oracle's insertion sort
// over the src -> dst path).  One lane.
__device__ __forceinline__ void nr_wide_branch_order(uint32_t *hops, int L, int border, const double *p)
{
    if (border == NR_BORDER_DST) {                          // walk order reversed
        for (int i = 0, j = L - 1; i < j; ++i, --j) { const uint32_t t = hops[i]; hops[i] = hops[j]; hops[j] = t; }
        return;
    }
    // s_i = hops[L-1-i] is the src -> dst path; sort it stably by p, then store it back reversed
    const bool desc = (border == NR_BORDER_P_DESC);
    for (int i = 1; i < L; ++i) {
        const uint32_t e = hops[L - 1 - i];
        const double pe = p[e];
        int j = i - 1;
        while (j >= 0 && (desc ? p[hops[L - 1 - j]] < pe : p[hops[L - 1 - j]] > pe)) {
            hops[L - 1 - (j + 1)] = hops[L - 1 - j];
            --j;
        }
        hops[L - 1 - (j + 1)] = e;
    }
}

// The learned branch order's scorer in a whole-GPU kernel: the weights, and the warp's scratch
// (nr_mlp_score_lanes: BF16 tiles, 16 outputs) in shared memory.
struct NrWideLearn {
    NrMlpDev M;
    uint32_t *scratch;
    float *y;
};

// Learned branch order of a path held dst side first in hops[0..L) (all lanes): the scorer
// estimates the residual reliability r of the subproblem with each UNKNOWN hop down (the
// features of the lane-group kernel's learned order: that child's edge-state fractions, the path
// length and the hop's place on it, p, the not-down degrees of src and dst less the hop, the
// masses, n and E), and the hops are branched largest (1 - p) x (1 - r) first -- a likely and
// critical failure first; ties keep path order (src side first); known hops go last (they make
// no child).  Keys go to v.order and the reordered hops through v.list (free after the search).
__device__ __forceinline__ void nr_wide_learned_order(const NrWideGraph &g, const NrWideView &v, uint32_t *hops,
                                                      int L, double mass, const NrWideLearn &W)
{
    constexpr uint32_t HM = (1u << NR_WIDE_HEAD_BITS) - 1u;
    const int lane = threadIdx.x & 31;
    const int n = g.n, E = g.e, src = g.src, dst = g.dst;
    const uint32_t *m = v.m;
    // the parent's UNKNOWN and up edges (mask bits past edge E-1 are padding)
    int unk = 0, up = 0;
    for (int k = lane; k < 4 * g.w4 && 16 * k < E; k += 32) {
        const int valid = min(16, E - 16 * k);
        const uint32_t vm = valid >= 16 ? 0x55555555u : ((1u << (2 * valid)) - 1u) & 0x55555555u;
        const uint32_t w = m[k], lo = w & vm, hi = (w >> 1) & vm;
        unk += __popc(lo & hi);
        up += __popc(lo & ~hi);
    }
    unk = __reduce_add_sync(NR_FULL, unk);
    up = __reduce_add_sync(NR_FULL, up);
    // not-down degrees of src and dst (their arc lists: in- or out-arcs, the same on undirected graphs)
    int ds = 0, dd = 0;
    for (int j = v.row[src] + lane; j < v.row[src + 1]; j += 32) {
        const uint32_t e = v.arc[j] >> NR_WIDE_HEAD_BITS;
        ds += (m[e >> 4] >> ((e & 15) << 1)) & 1u;
    }
    for (int j = v.row[dst] + lane; j < v.row[dst + 1]; j += 32) {
        const uint32_t e = v.arc[j] >> NR_WIDE_HEAD_BITS;
        dd += (m[e >> 4] >> ((e & 15) << 1)) & 1u;
    }
    ds = __reduce_add_sync(NR_FULL, ds);
    dd = __reduce_add_sync(NR_FULL, dd);
    (void)HM;
    float *key = reinterpret_cast<float *>(v.order);
    const float inv_e = E > 0 ? 1.f / (float)E : 0.f, inv_n1 = n > 1 ? 1.f / (float)(n - 1) : 0.f;
    for (int c = 0; c < L; c += 32) {
        const int k = c + lane;
        const uint32_t e = k < L ? hops[k] : 0u;
        const bool has = k < L && ((m[e >> 4] >> ((e & 15) << 1)) & 3u) == 3u;
        float f[NR_MLP_IN];
        const double pe = has ? v.p[e] : 0.0;
        const int pos = L - 1 - k;                          // place on the path, src side first
        {
            const double cm = mass * (1.0 - pe);
            const int dsx = ds - (pos == 0 ? 1 : 0), ddx = dd - (pos == L - 1 ? 1 : 0);
            f[0] = cm > 0.0 ? fmaxf(log2f((float)cm) * (1.f / 64.f), -16.f) : -16.f;   // below FLT_MIN: -16
            f[1] = (unk - 1) * inv_e;
            f[2] = up * inv_e;
            f[3] = (E - unk - up + 1) * inv_e;
            f[4] = (float)L / (float)n;
            f[5] = (float)(pos + 1) / (float)L;
            f[6] = (float)pe;
            f[7] = dsx * inv_n1;
            f[8] = ddx * inv_n1;
            f[9] = min(dsx, ddx) * inv_n1;
            f[10] = mass > 0.0 ? fmaxf(log2f((float)mass) * (1.f / 64.f), -16.f) : -16.f;
            f[11] = n * (1.f / 64.f);
            f[12] = E * (1.f / 512.f);
            f[13] = 0.f;
            f[14] = 0.f;
            f[15] = 1.f;
        }
        float r = nr_mlp_score_lanes(W.M, W.scratch, W.y, has, f);
        r = (r >= 0.f) ? fminf(r, 1.f) : 0.f;            // a NaN estimate must not break the ranking
        if (k < L) key[k] = has ? (1.f - (float)pe) * (1.f - r) : -1.f;
    }
    __syncwarp();
    // rank of hop k: the hops with a larger key, or an equal key nearer src, go first; the walk
    // branches hops[L-1] first, so rank r goes to hops[L-1-r]
    uint32_t *nh = v.list;
    for (int k = lane; k < L; k += 32) {
        const float kk = key[k];
        int r = 0;
        for (int j = 0; j < L; ++j) {
            const float kj = key[j];
            r += (kj > kk || (kj == kk && j > k)) ? 1 : 0;  // j > k: nearer src
        }
        nh[L - 1 - r] = hops[k];
    }
    __syncwarp();
    for (int k = lane; k < L; k += 32) hops[k] = nh[k];
    __syncwarp();
}

template <int W4>
__device__ __forceinline__ void nr_wide_step(const NrWideGraph &g, const NrWideView &v, double mass, double eps,
                                             const NrWideOut &O, NrWideAcc &A, bool fork = false, int border = 0,
                                             const NrWideLearn *learn = nullptr)
{
    constexpr int NW = 4 * W4;
    const int lane = threadIdx.x & 31;
    const int n = g.n, src = g.src, dst = g.dst;
    uint32_t *m = v.m, *par = v.par, *hops = v.hops;
    if (lane == 0) {
        A.nodes++;
        nr_fix_sub(A.net, nr_fix_of(mass));
    }
    __syncwarp();
    if (eps > 0.0 && mass < eps) {          // main.cu:537-543
        if (lane == 0) { A.trunc++; nr_fix_add_mass(A.et, mass); }
        __syncwarp();
        return;
    }
    if (fork && nr_wide_bfs(g, v, true)) {   // connected: the whole mass to R
        if (lane == 0) { A.leaves++; nr_fix_add_mass(A.R, mass); }
        __syncwarp();
        return;
    }
    int no = 0;
    const bool found = g.bitset ? nr_wide_bfs_bits(g, v) : nr_wide_bfs(g, v, false, g.nk ? &no : nullptr);
    int L = 0;
    if (!found) {
        if (lane == 0) A.dead++;
        __syncwarp();
        return;
    }
    if (g.bitset) {
        L = nr_wide_path_bits(g, v, hops);
        if (lane == 0 && border != NR_BORDER_SRC && border != NR_BORDER_LEARNED && L > 1)
            nr_wide_branch_order(hops, L, border, v.p);
    } else if (lane == 0) {
        if (g.nk) {
            // K-terminal: the tree of the terminals' parent paths to src (marked in NF), its
            // edges in visit order, stored last first as the path hops are (dst side first)
            uint32_t *mk = v.NF;
            for (int i = 0; i < g.nwd; ++i) mk[i] = 0u;
            for (int i = 1; i < no; ++i) {
                const int t = (int)v.order[i];
                if (!((v.kmask[t >> 5] >> (t & 31)) & 1u)) continue;
                for (int x = t; x != src && !((mk[x >> 5] >> (x & 31)) & 1u); x = (int)(par[x] >> 16))
                    mk[x >> 5] |= 1u << (x & 31);
            }
            int cntm = 0;
            for (int i = 1; i < no; ++i) cntm += (mk[v.order[i] >> 5] >> (v.order[i] & 31)) & 1u;
            int j = 0;
            for (int i = 1; i < no; ++i) {
                const int x = (int)v.order[i];
                if ((mk[x >> 5] >> (x & 31)) & 1u) hops[cntm - 1 - j++] = par[x] & 0xffffu;
            }
            L = cntm;
        } else {
            // ---- path: hops[] from dst back to src (L hops) ----
            int x = dst, h = 0;
            while (x != src && h < n) {
                const uint32_t pe = par[x];
                hops[h++] = pe & 0xffffu;
                x = (int)(pe >> 16);
            }
            L = h;
            if (border != NR_BORDER_SRC && border != NR_BORDER_LEARNED && L > 1)
                nr_wide_branch_order(hops, L, border, v.p);
        }
    }
    L = __shfl_sync(NR_FULL, L, 0);
    __syncwarp();
    if (learn && border == NR_BORDER_LEARNED && L > 1 && !g.nk) nr_wide_learned_order(g, v, hops, L, mass, *learn);
    if (fork) {
        // the pivot: largest p among the UNKNOWN hops, the nearest dst (lowest index) on ties
        double bp = -1.0;
        int bh = 1 << 30;
        for (int h = lane; h < L; h += 32) {
            const uint32_t e = hops[h];
            if (((m[e >> 4] >> ((e & 15) << 1)) & 3u) == 3u) {
                const double pe = v.p[e];
                if (pe > bp || (pe == bp && h < bh)) { bp = pe; bh = h; }
            }
        }
        for (int off = 16; off > 0; off >>= 1) {
            const double op = __shfl_xor_sync(NR_FULL, bp, off);
            const int oh = __shfl_xor_sync(NR_FULL, bh, off);
            if (op > bp || (op == bp && oh < bh)) { bp = op; bh = oh; }
        }
        if (bp < 0.0) {                 // not reached: without a path of up edges one hop is UNKNOWN
            if (lane == 0) { A.leaves++; nr_fix_add_mass(A.R, mass); }
            __syncwarp();
            return;
        }
        const int e = (int)hops[bh];
        unsigned long long base = 0;
        if (lane == 0) base = atomicAdd(O.count, 2ull);
        base = __shfl_sync(NR_FULL, base, 0);
        const int sh = (e & 15) << 1;
        nr_wide_emit(O, A, m, g.w4, base, e, 3u << sh, __dmul_rn(mass, __dsub_rn(1.0, v.p[e])));   // down
        nr_wide_emit(O, A, m, g.w4, base + 1, e, 2u << sh, __dmul_rn(mass, v.p[e]));    // up
        __syncwarp();
        return;
    }
    // number of UNKNOWN hops -> one slot range for all children
    int unk = 0;
    for (int h = lane; h < L; h += 32) {
        const uint32_t e = hops[h];
        unk += ((m[e >> 4] >> ((e & 15) << 1)) & 3u) == 3u;
    }
    for (int off = 16; off > 0; off >>= 1) unk += __shfl_xor_sync(NR_FULL, unk, off);
    unsigned long long base = 0;
    if (lane == 0 && unk > 0) base = atomicAdd(O.count, (unsigned long long)unk);
    base = __shfl_sync(NR_FULL, base, 0);
    // children in hop order, src side first; lanes own mask words (in registers when the width
    // is compiled in, else in the warp's working copy wk)
    const int w4 = W4 ? W4 : g.w4;
    uint32_t w0 = 0u, w1 = 0u;
    if (W4) {
        w0 = (lane < NW) ? m[lane] : 0u;
        w1 = (lane + 32 < NW) ? m[lane + 32] : 0u;
    } else {
        for (int i = lane; i < 4 * w4; i += 32) v.wk[i] = m[i];
        __syncwarp();
    }
    double Pm = mass;
    int k = 0;
    for (int h = L - 1; h >= 0; --h) {
        const uint32_t e = hops[h];
        const int sh = (int)(e & 15u) << 1;
        const int wi = (int)(e >> 4);
        if (((m[wi] >> sh) & 3u) != 3u) continue;          // only UNKNOWN hops branch
        const unsigned long long slot = base + (unsigned long long)k;
        const double cm = __dmul_rn(Pm, __dsub_rn(1.0, v.p[e]));
        if (slot < O.cap) {
            uint32_t *dstw = reinterpret_cast<uint32_t *>(O.mask + slot * w4);
            if (W4) {
                if (lane < NW) __stcg(dstw + lane, (lane == wi) ? (w0 & ~(3u << sh)) : w0);
                if (lane + 32 < NW) __stcg(dstw + lane + 32, (lane + 32 == wi) ? (w1 & ~(3u << sh)) : w1);
            } else {
                for (int i = lane; i < 4 * w4; i += 32) __stcg(dstw + i, (i == wi) ? (v.wk[i] & ~(3u << sh)) : v.wk[i]);
            }
            if (lane == 0) {
                __stcg(O.mass + slot, cm);
                nr_fix_add_mass(A.net, cm);
                if (O.key) {
                    const int b = nr_bucket(cm, O.shift, O.nb);
                    __stcg(O.key + slot, (unsigned char)b);
                    atomicAdd(&O.hist[b], 1u);
                }
            }
        } else if (lane == 0) {                             // queue full (main.cu:245-252)
            A.spilled++;
            nr_fix_add_mass(A.es, cm);
        }
        if (W4) {                                           // this hop is up in later children
            if (lane == wi) w0 &= ~(2u << sh);
            if (lane + 32 == wi) w1 &= ~(2u << sh);
        } else {
            __syncwarp();
            if (lane == 0) v.wk[wi] &= ~(2u << sh);
            __syncwarp();
        }
        Pm = __dmul_rn(Pm, v.p[e]);
        ++k;
    }
    if (lane == 0) { A.leaves++; nr_fix_add_mass(A.R, Pm); }
    __syncwarp();
}

__device__ __forceinline__ void nr_wide_acc_init(NrWideAcc &A)
{
    A.R = A.et = A.es = nr_fix_zero();
    // the root is queued before the first wave: block 0's first lane holds its mass
    A.net = (blockIdx.x == 0 && threadIdx.x == 0) ? nr_fix_of(1.0) : nr_fix_zero();
    A.nodes = A.leaves = A.dead = A.trunc = A.spilled = 0;
}

// The block's partial sums from its warps' accumulators (lane 0 of each warp holds them).
__device__ __forceinline__ void nr_wide_block_partial(NrPartial *out, const NrWideAcc &A)
{
    NrWideAcc F;
    if ((threadIdx.x & 31) == 0) F = A;
    else nr_wide_acc_init(F);                                // zeros off thread 0
    nr_block_partial(out, F.R, F.et, F.es, F.net, F.nodes, F.leaves, F.dead, F.trunc, F.spilled);
}

// Sum over the block of a per-thread count, on every thread.
__device__ __forceinline__ unsigned long long nr_block_u64_sum(unsigned long long x)
{
    __shared__ unsigned long long s_x[32];
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(NR_FULL, x, off);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s_x[threadIdx.x >> 5] = x;
    __syncthreads();
    unsigned long long t = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += s_x[i];
    return t;
}

// This block's share of the stop test after a wave (all threads call it).
__device__ __forceinline__ void nr_wide_write_share(NrWideShare *slot, const NrWideAcc &A, int bid = -1)
{
    if (bid < 0) bid = (int)blockIdx.x;
    NrFix w = nr_fix_zero();
    unsigned long long nodes = 0;
    if ((threadIdx.x & 31) == 0) {
        w = A.et;
        nr_fix_add(w, A.es);
        nr_fix_add(w, A.net);
        nodes = A.nodes;
    }
    w = nr_block_fix_sum(w);
    nodes = nr_block_u64_sum(nodes);
    if (threadIdx.x == 0) {
        NrWideShare *d = slot + bid;
        __stcg(&d->width.w0, w.w0);
        __stcg(&d->width.w1, w.w1);
        __stcg(&d->width.w2, w.w2);
        __stcg(&d->nodes, nodes);
    }
}

// Stop test before a wave from the shares of the last one (every block gets
// the same answer): 0 go on, 1 target width met, 3 node budget reached.
__device__ __forceinline__ int nr_wide_stop_test(const NrWideShare *slot, bool first, int target_on,
                                                 const NrFix &target_fix, unsigned long long max_nodes,
                                                 unsigned nblk = 0)
{
    if (nblk == 0) nblk = gridDim.x;
    if (!target_on && !max_nodes) return 0;
    NrFix width = nr_fix_zero();
    unsigned long long nodes = 0;
    if (first) {
        if (threadIdx.x == 0) width = nr_fix_of(1.0);      // the root alone is queued
    } else {
        for (unsigned b = threadIdx.x; b < nblk; b += blockDim.x) {
            NrFix v;                                       // written by other blocks: read from L2
            v.w0 = __ldcg(&slot[b].width.w0);
            v.w1 = __ldcg(&slot[b].width.w1);
            v.w2 = __ldcg(&slot[b].width.w2);
            nr_fix_add(width, v);
            nodes += __ldcg(&slot[b].nodes);
        }
    }
    width = nr_block_fix_sum(width);
    nodes = nr_block_u64_sum(nodes);
    if (target_on && nr_fix_le(width, target_fix)) return 1;
    if (max_nodes && nodes >= max_nodes) return 3;
    return 0;
}

template <int W4>
__global__ void __launch_bounds__(NR_WIDE_BLOCK, 6) nr_grid_wide_kernel(NrGridWideParams P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const NrWideGraph g = P.g;
    if (!g.tables_global) nr_stage_blob(smem, P.blob, g.blob_bytes);
    __syncthreads();
    const NrWideView v = nr_wide_view(smem, P.blob, g);
    const int w4 = W4 ? W4 : g.w4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long gw = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + warp;
    const unsigned long long TW = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long cap = P.capacity;
    // the warp's accumulators: shared memory, written by its lane 0 only (registers for the step)
    __shared__ NrWideAcc s_acc[NR_WIDE_BLOCK / 32];
    NrWideAcc &A = s_acc[warp];
    if (lane == 0) nr_wide_acc_init(A);
    __syncwarp();

    for (int wave = 0; wave < P.max_waves; ++wave) {
        unsigned long long n_in = *(volatile unsigned long long *)&P.wave_count[wave];
        if (n_in > cap) n_in = cap;
        if (n_in == 0) break;
        const int stop = nr_wide_stop_test(P.wpart + (size_t)((wave + 1) & 1) * gridDim.x, wave == 0,
                                           P.target_on, P.target_fix, P.max_nodes);
        if (stop) {
            if (threadIdx.x == 0 && blockIdx.x == 0) { P.stop_wave[0] = wave; P.stop_wave[1] = stop; }
            break;
        }
        const uint4 *in_mask = P.mask[wave & 1];
        const double *in_mass = P.mass[wave & 1];
        NrWideOut O;
        O.mask = P.mask[(wave + 1) & 1];
        O.mass = P.mass[(wave + 1) & 1];
        O.key = nullptr;
        O.count = &P.wave_count[wave + 1];
        O.cap = cap;
        O.shift = 0;
        O.nb = 1;
        O.hist = nullptr;
        for (unsigned long long idx = gw; idx < n_in; idx += TW) {
            nr_wide_load_mask(v.m, in_mask + idx * w4, w4);
            const double mass = __ldcg(in_mass + idx);
            __syncwarp();
            nr_wide_step<W4>(g, v, mass, P.eps, O, A, P.fork != 0, P.border);
        }
        if (P.target_on || P.max_nodes) nr_wide_write_share(P.wpart + (size_t)(wave & 1) * gridDim.x, A);
        if (!nr_grid_sync(P.bar_count, P.bar_gen, P.status, P.timeout_ns)) break;
        if (wave + 1 == P.max_waves && threadIdx.x == 0 && blockIdx.x == 0 &&
            *(volatile unsigned long long *)&P.wave_count[wave + 1] != 0)
            atomicOr(P.status, NR_DEV_ERR_WAVES);
    }
    nr_wide_block_partial(P.partials + blockIdx.x, A);
}

// Several instances in one cooperative launch, breadth-first waves: instance i owns the
// blocks [i * bpi, (i + 1) * bpi) and runs nr_grid_wide_kernel's loop on them -- its own
// ping-pong buffers, wave counters, barrier, stop-test shares and stop record -- so every
// instance follows the one-instance schedule exactly, and the instances of a batch of large
// graphs run side by side instead of one launch each.
struct NrGridWideMultiParams {
    const NrWideGraph *g;            // [m] in global memory
    const unsigned char *blob;       // the instances' tables, instance i at blob_off[i]
    const long long *blob_off;       // [m]
    const uint4 *root;               // [m][w4]: the instances' root masks
    uint4 *mask;                     // [m][2][mask_half]: an instance's two wave buffers
    double *mass;                    // [m][2][mass_half]
    unsigned long long mask_half;    // 16-byte blocks of one wave buffer (capacity x the widest mask)
    unsigned long long mass_half;    // masses of one wave buffer (capacity, rounded up)
    unsigned long long capacity;
    unsigned long long *wave_count;  // [m][max_waves + 1]
    int max_waves;
    unsigned *bar;                   // [m][4]: barrier count, generation, status
    NrPartial *partials;             // [gridDim.x]
    NrWideShare *wpart;              // [m][2][bpi]
    int *stop_wave;                  // [m][2]: waves run before a stop (or -1), stop reason
    int m, bpi;
    double eps;
    long long timeout_ns;
    int target_on;
    NrFix target_fix;
    unsigned long long max_nodes;
    int border;
};

template <int W4>
__global__ void __launch_bounds__(NR_WIDE_BLOCK, 6) nr_grid_wide_multi_kernel(NrGridWideMultiParams P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    const int inst = (int)blockIdx.x / P.bpi, lb = (int)blockIdx.x % P.bpi;
    const NrWideGraph g = P.g[inst];
    const unsigned char *blob = P.blob + P.blob_off[inst];
    if (!g.tables_global) nr_stage_blob(smem, blob, g.blob_bytes);
    __syncthreads();
    const NrWideView v = nr_wide_view(smem, blob, g);
    const int w4 = W4 ? W4 : g.w4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long gw = (unsigned long long)lb * (blockDim.x >> 5) + warp;
    const unsigned long long TW = (unsigned long long)P.bpi * (blockDim.x >> 5);
    const unsigned long long cap = P.capacity;
    uint4 *mask0 = P.mask + (size_t)inst * 2 * P.mask_half;
    double *mass0 = P.mass + (size_t)inst * 2 * P.mass_half;
    unsigned long long *wave_count = P.wave_count + (size_t)inst * (P.max_waves + 1);
    unsigned *bar = P.bar + (size_t)inst * 4;
    int *status = reinterpret_cast<int *>(bar + 2);
    NrWideShare *wpart = P.wpart + (size_t)inst * 2 * P.bpi;
    int *stop_wave = P.stop_wave + (size_t)inst * 2;
    __shared__ NrWideAcc s_acc[NR_WIDE_BLOCK / 32];        // as in nr_grid_wide_kernel
    NrWideAcc &A = s_acc[warp];
    if (lane == 0) {
        nr_wide_acc_init(A);
        // the root is queued before the first wave: the instance's first block holds its mass
        A.net = (lb == 0 && threadIdx.x == 0) ? nr_fix_of(1.0) : nr_fix_zero();
    }
    __syncwarp();
    // the instance's first block queues its root (mass 1) and clears its stop record; the group
    // meets once before the first wave
    if (lb == 0 && warp == 0) {
        for (int k = lane; k < w4; k += 32) mask0[k] = P.root[(size_t)inst * w4 + k];
        if (lane == 0) {
            mass0[0] = 1.0;
            wave_count[0] = 1ull;
            stop_wave[0] = -1;
            stop_wave[1] = 0;
        }
    }
    bool ok = nr_grid_sync(bar, bar + 1, status, P.timeout_ns, (unsigned)P.bpi);

    for (int wave = 0; ok && wave < P.max_waves; ++wave) {
        unsigned long long n_in = *(volatile unsigned long long *)&wave_count[wave];
        if (n_in > cap) n_in = cap;
        if (n_in == 0) break;
        const int stop = nr_wide_stop_test(wpart + (size_t)((wave + 1) & 1) * P.bpi, wave == 0, P.target_on,
                                           P.target_fix, P.max_nodes, (unsigned)P.bpi);
        if (stop) {
            if (threadIdx.x == 0 && lb == 0) { stop_wave[0] = wave; stop_wave[1] = stop; }
            break;
        }
        const uint4 *in_mask = mask0 + (size_t)(wave & 1) * P.mask_half;
        const double *in_mass = mass0 + (size_t)(wave & 1) * P.mass_half;
        NrWideOut O;
        O.mask = mask0 + (size_t)((wave + 1) & 1) * P.mask_half;
        O.mass = mass0 + (size_t)((wave + 1) & 1) * P.mass_half;
        O.key = nullptr;
        O.count = &wave_count[wave + 1];
        O.cap = cap;
        O.shift = 0;
        O.nb = 1;
        O.hist = nullptr;
        for (unsigned long long idx = gw; idx < n_in; idx += TW) {
            nr_wide_load_mask(v.m, in_mask + idx * w4, w4);
            const double mass = __ldcg(in_mass + idx);
            __syncwarp();
            nr_wide_step<W4>(g, v, mass, P.eps, O, A, false, P.border);
        }
        if (P.target_on || P.max_nodes) nr_wide_write_share(wpart + (size_t)(wave & 1) * P.bpi, A, lb);
        if (!nr_grid_sync(bar, bar + 1, status, P.timeout_ns, (unsigned)P.bpi)) break;
        if (wave + 1 == P.max_waves && threadIdx.x == 0 && lb == 0 &&
            *(volatile unsigned long long *)&wave_count[wave + 1] != 0)
            atomicOr(status, NR_DEV_ERR_WAVES);
    }
    nr_wide_block_partial(P.partials + blockIdx.x, A);
}

// Records queued in all buckets and the highest non-empty bucket (every block
// reads the same counters after a grid barrier and gets the same answer).
__device__ __forceinline__ void nr_bucket_select(const unsigned long long *bcount, int nb, int *b_out,
                                                 unsigned long long *live_out)
{
    __shared__ int s_b[32];
    int bmin = 1 << 30;
    unsigned long long c = 0;
    for (int b = threadIdx.x; b < nb; b += blockDim.x) {
        const unsigned long long x = __ldcg(bcount + b);
        c += x;
        if (x && b < bmin) bmin = b;
    }
    for (int off = 16; off > 0; off >>= 1) bmin = min(bmin, __shfl_xor_sync(NR_FULL, bmin, off));
    *live_out = nr_block_u64_sum(c);        // (its barriers also order s_b's reuse)
    if ((threadIdx.x & 31) == 0) s_b[threadIdx.x >> 5] = bmin;
    __syncthreads();
    int bb = 1 << 30;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) bb = min(bb, s_b[i]);
    *b_out = bb;
}

// In-place compaction of the arena's first `used` slots: the `live` records
// end up in slots [0, live).  Free slots below `live` are paired, in slot
// order, with records at or above it (there are as many of each).  Three
// grid barriers; false if one of them failed.
template <int W4>
__device__ __forceinline__ bool nr_bucket_compact(const NrBucketWideParams &P, unsigned long long used,
                                                  unsigned long long live)
{
    __shared__ unsigned long long s_h[NR_WIDE_BLOCK / 32], s_l[NR_WIDE_BLOCK / 32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    // block b owns slots [b * chunk, (b + 1) * chunk), each warp a contiguous part of them
    const unsigned long long chunk = ((used + gridDim.x - 1) / gridDim.x + 31) & ~31ull;
    const unsigned long long sub = ((chunk + nwarp - 1) / nwarp + 31) & ~31ull;
    const unsigned long long c0 = (unsigned long long)blockIdx.x * chunk;
    const unsigned long long c1 = min(used, c0 + chunk);
    const unsigned long long w0 = c0 + (unsigned long long)warp * sub;
    const unsigned long long w1 = min(c1, w0 + sub);
    const unsigned long long iters = (w1 > w0) ? (w1 - w0 + 31) / 32 : 0;
    unsigned long long nh = 0, nl = 0;      // free slots below live, records at or above it
    for (unsigned long long it = 0; it < iters; ++it) {
        const unsigned long long s = w0 + it * 32 + lane;
        const unsigned k = (s < w1) ? __ldcg(P.key + s) : NR_WIDE_FREE;
        nh += __popc(__ballot_sync(NR_FULL, s < w1 && s < live && k == NR_WIDE_FREE));
        nl += __popc(__ballot_sync(NR_FULL, s < w1 && s >= live && k != NR_WIDE_FREE));
    }
    if (lane == 0) { s_h[warp] = nh; s_l[warp] = nl; }
    __syncthreads();
    if (threadIdx.x == 0) {
        unsigned long long th = 0, tl = 0;
        for (int i = 0; i < nwarp; ++i) { th += s_h[i]; tl += s_l[i]; }
        __stcg(P.ccount + blockIdx.x, th);
        __stcg(P.ccount + gridDim.x + blockIdx.x, tl);
    }
    if (!nr_grid_sync(P.bar_count, P.bar_gen, P.status, P.timeout_ns)) return false;
    // global ranks: earlier blocks, then earlier warps of this block, then earlier lanes
    unsigned long long rh = 0, rl = 0, moved = 0;
    for (unsigned b = 0; b < gridDim.x; ++b) {
        const unsigned long long h = __ldcg(P.ccount + b);
        if (b < blockIdx.x) { rh += h; rl += __ldcg(P.ccount + gridDim.x + b); }
        moved += h;
    }
    for (int i = 0; i < warp; ++i) { rh += s_h[i]; rl += s_l[i]; }
    unsigned *hole = P.list, *from = P.list + P.capacity / 2;
    for (unsigned long long it = 0; it < iters; ++it) {
        const unsigned long long s = w0 + it * 32 + lane;
        const unsigned k = (s < w1) ? __ldcg(P.key + s) : NR_WIDE_FREE;
        const unsigned mh = __ballot_sync(NR_FULL, s < w1 && s < live && k == NR_WIDE_FREE);
        const unsigned ml = __ballot_sync(NR_FULL, s < w1 && s >= live && k != NR_WIDE_FREE);
        const unsigned below = (1u << lane) - 1u;
        if ((mh >> lane) & 1u) __stcg(hole + rh + __popc(mh & below), (unsigned)s);
        if ((ml >> lane) & 1u) __stcg(from + rl + __popc(ml & below), (unsigned)s);
        rh += __popc(mh);
        rl += __popc(ml);
    }
    if (!nr_grid_sync(P.bar_count, P.bar_gen, P.status, P.timeout_ns)) return false;
    // one warp per moved record; sources (>= live) and destinations (< live) never overlap
    const unsigned long long gw = (unsigned long long)blockIdx.x * nwarp + warp;
    const unsigned long long TW = (unsigned long long)gridDim.x * nwarp;
    for (unsigned long long r = gw; r < moved; r += TW) {
        const unsigned long long d = __ldcg(hole + r), s = __ldcg(from + r);
        const int w4 = W4 ? W4 : P.g.w4;
        for (int k = lane; k < w4; k += 32) __stcg(P.mask + d * w4 + k, __ldcg(P.mask + s * w4 + k));
        if (lane == 0) {
            __stcg(P.mass + d, __ldcg(P.mass + s));
            __stcg(P.key + d, __ldcg(P.key + s));
        }
    }
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        *P.top = live;
        P.stop_info[2]++;
    }
    return nr_grid_sync(P.bar_count, P.bar_gen, P.status, P.timeout_ns);
}

// per warp, after the block's search scratch: the scorer's tiles and outputs (LEARN)
#define NR_WIDE_LEARN_WORDS (NR_MLP_WARP_WORDS + 16)

// ---- one lane per subproblem (the bucketed queue's LANES instantiation) ----
// Undirected simple graphs of <= 250 nodes with the bit-set tables (whose in-arc lists are then
// every node's neighbours), two-terminal path branching, the src-side-first branch order.  A warp
// step expands 32 records of the wave, one a lane, where nr_wide_step gives each record the whole
// warp.  A lane's scratch, in shared memory as [row][lane] columns after the block's search
// scratch: the record's mask words, each node's BFS level (a byte; 0xff unseen) and the BFS
// queue (node bytes), whose first L + 1 bytes then hold the path's nodes, src first.
#define NR_WIDE_LANES_MAX_N 250
// A wave runs one lane a record from this many records a warp up, else a warp a record.  RGG
// N=200 (bucketed queue, 1 M / 20 M subproblems): 1, 4, 8, 16, 32, never: 19.5 / 186.5, 17.9 /
// 185.1, 17.1 / 184.3, 17.3 / 184.8, 19.3 / 186.9, 29.2 / 521 ms; the warp-per-subproblem
// kernel, whose registers and shared memory allow three times the blocks: 18.2 / 255 ms.
#define NR_WIDE_LANE_MIN_PER_WARP 8
__host__ __device__ inline size_t nr_wide_lane_shm(int n, int w4)
{
    return (size_t)(4 * w4 + 2 * ((n + 3) / 4)) * 32 * 4;
}

struct NrWideLaneAcc {
    NrFix R, et, es, net;
    unsigned long long nodes, leaves, dead, trunc, spilled;
};

__device__ __forceinline__ void nr_wide_lane_acc_zero(NrWideLaneAcc &a)
{
    a.R = a.et = a.es = a.net = nr_fix_zero();
    a.nodes = a.leaves = a.dead = a.trunc = a.spilled = 0;
}

// The lanes' sums and counts into the warp's accumulators (all lanes call; lane 0 adds).
__device__ __forceinline__ void nr_wide_lane_fold(NrWideLaneAcc &a, NrWideAcc &A)
{
    const NrFix R = nr_fix_warp_sum(a.R), net = nr_fix_warp_sum(a.net);
    const NrFix et = nr_fix_warp_sum_sparse(a.et), es = nr_fix_warp_sum_sparse(a.es);
    const unsigned long long nodes = nr_warp_sum_u64r(a.nodes), leaves = nr_warp_sum_u64r(a.leaves);
    const unsigned long long dead = nr_warp_sum_u64r(a.dead), trunc = nr_warp_sum_u64r(a.trunc);
    const unsigned long long spilled = nr_warp_sum_u64r(a.spilled);
    if ((threadIdx.x & 31) == 0) {
        nr_fix_add(A.R, R); nr_fix_add(A.et, et); nr_fix_add(A.es, es); nr_fix_add(A.net, net);
        A.nodes += nodes; A.leaves += leaves; A.dead += dead; A.trunc += trunc; A.spilled += spilled;
    }
    __syncwarp();
    nr_wide_lane_acc_zero(a);
}

// One lane's record (all lanes call: the children's slots are one warp-wide allocation).  mc:
// the lane's mask column (word k at mc[32 k]); dq: its level and queue columns (byte i at
// dq[32 i] and dq[32 (4 DB + i)]).  The search, path, children and products are nr_wide_step's
// for these graphs: a level BFS over the not-down edges, the parent of a node on level l + 1 the
// smallest node of level l adjacent to it, one child per UNKNOWN path edge src side first.
template <int W4>
__device__ __forceinline__ void nr_wide_lane_step(const NrWideGraph &g, const NrWideView &v, uint32_t *mc,
                                                  unsigned char *dq, bool valid, double mass, double eps,
                                                  const NrWideOut &O, NrWideLaneAcc &A, int *status)
{
    constexpr uint32_t HM = (1u << NR_WIDE_HEAD_BITS) - 1u;
    const int lane = threadIdx.x & 31;
    const int n = g.n, src = g.src, dst = g.dst;
    unsigned char *lev = dq;
    unsigned char *que = dq + (size_t)((n + 3) / 4) * 4 * 32;
    auto state = [&](int e) -> uint32_t { return (mc[32 * (e >> 4)] >> ((e & 15) << 1)) & 3u; };
    bool active = valid;
    if (valid) {
        A.nodes++;
        nr_fix_sub(A.net, nr_fix_of(mass));
        if (eps > 0.0 && mass < eps) {                      // main.cu:537-543
            A.trunc++;
            nr_fix_add_mass(A.et, mass);
            active = false;
        }
    }
    int L = -1, nch = 0;                                    // L < 0: no path
    bool bad = false;
    if (active) {
        for (int i = 0; i < n; ++i) lev[32 * i] = 0xff;
        if (src == dst) {
            L = 0;
        } else {
            lev[32 * src] = 0;
            que[0] = (unsigned char)src;
            int head = 0, tail = 1;
            bool found = false;
            while (!found && head < tail) {                 // each node is queued once: <= n pops
                const int u = que[32 * head++];
                const int du = lev[32 * u];
                for (int j = v.row[u], je = v.row[u + 1]; j < je; ++j) {
                    const uint32_t a = v.arc[j];
                    const int e = (int)(a >> NR_WIDE_HEAD_BITS), w = (int)(a & HM);
                    if (state(e) == NR_EDGE_DOWN || lev[32 * w] != 0xff) continue;
                    lev[32 * w] = (unsigned char)(du + 1);
                    que[32 * tail++] = (unsigned char)w;
                    if (w == dst) { found = true; break; }
                }
            }
            if (found) {
                L = lev[32 * dst];
                que[32 * L] = (unsigned char)dst;           // the path's nodes, src first
                int x = dst;
                for (int l = L - 1; l >= 0 && !bad; --l) {
                    int best = n, be = -1;
                    for (int j = v.row[x], je = v.row[x + 1]; j < je; ++j) {
                        const uint32_t a = v.arc[j];
                        const int e = (int)(a >> NR_WIDE_HEAD_BITS), w = (int)(a & HM);
                        if (lev[32 * w] != l || state(e) == NR_EDGE_DOWN) continue;
                        if (w < best) { best = w; be = e; }
                    }
                    if (be < 0) { bad = true; break; }
                    nch += state(be) == NR_EDGE_UNKNOWN;
                    que[32 * l] = (unsigned char)best;
                    x = best;
                }
                if (!bad && x != src) bad = true;
            }
        }
    }
    if (bad) {                                              // an internal check failed: no children
        atomicOr(status, NR_DEV_ERR_BOUNDS);
        nch = 0;
        L = -1;
        active = false;
    }
    // the warp's children take one range of slots
    int pre = nch;
#pragma unroll
    for (int off = 1; off < 32; off <<= 1) {
        const int t = __shfl_up_sync(NR_FULL, pre, off);
        if (lane >= off) pre += t;
    }
    const int total = __shfl_sync(NR_FULL, pre, 31);
    unsigned long long base = 0;
    if (lane == 0 && total > 0) base = atomicAdd(O.count, (unsigned long long)total);
    base = __shfl_sync(NR_FULL, base, 0);
    unsigned long long q = base + (unsigned long long)(pre - nch);
    if (L < 0) {
        if (active) A.dead++;
        return;
    }
    double Pm = mass;
    for (int h = 0; h < L; ++h) {
        const int u = que[32 * h], x = que[32 * (h + 1)];
        int e = 0;
        for (int j = v.row[x], je = v.row[x + 1]; j < je; ++j)
            if ((int)(v.arc[j] & HM) == u) { e = (int)(v.arc[j] >> NR_WIDE_HEAD_BITS); break; }
        const int wi = e >> 4, sh = (e & 15) << 1;
        const uint32_t wv = mc[32 * wi];
        if (((wv >> sh) & 3u) != 3u) continue;              // only UNKNOWN hops branch
        const double pe = v.p[e];
        const double cm = __dmul_rn(Pm, __dsub_rn(1.0, pe));
        Pm = __dmul_rn(Pm, pe);
        if (q < O.cap) {
            uint4 *d = O.mask + q * W4;
#pragma unroll
            for (int kk = 0; kk < W4; ++kk) {
                uint32_t r[4];
#pragma unroll
                for (int i = 0; i < 4; ++i) {
                    const int k = 4 * kk + i;
                    r[i] = (k == wi) ? (wv & ~(3u << sh)) : mc[32 * k];
                }
                __stcg(d + kk, make_uint4(r[0], r[1], r[2], r[3]));
            }
            __stcg(O.mass + q, cm);
            nr_fix_add_mass(A.net, cm);
            if (O.key) {
                const int b = nr_bucket(cm, O.shift, O.nb);
                __stcg(O.key + q, (unsigned char)b);
                atomicAdd(&O.hist[b], 1u);
            }
        } else {                                            // queue full (main.cu:245-252)
            A.spilled++;
            nr_fix_add_mass(A.es, cm);
        }
        mc[32 * wi] = wv & ~(2u << sh);                     // this hop is up in later children
        ++q;
    }
    A.leaves++;
    nr_fix_add_mass(A.R, Pm);
}

// LEARN: the learned branch order (NR_BORDER_LEARNED), with the scorer's scratch per warp.
// LANES: one lane per subproblem (nr_wide_lane_step), with its scratch per warp.
template <int W4, bool LEARN = false, bool LANES = false>
__global__ void __launch_bounds__(NR_WIDE_BLOCK, LEARN ? 3 : LANES ? 2 : 6) nr_bucket_wide_kernel(NrBucketWideParams P)
{
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ unsigned s_hist[NR_WIDE_MAX_NB + 1];
    const NrWideGraph g = P.g;
    if (!g.tables_global) nr_stage_blob(smem, P.blob, g.blob_bytes);
    __syncthreads();
    const NrWideView v = nr_wide_view(smem, P.blob, g);
    NrWideLearn W;
    if constexpr (LEARN) {
        uint32_t *ls = reinterpret_cast<uint32_t *>(smem + nr_wide_block_shm(g, (int)(blockDim.x >> 5))) +
                       (size_t)(threadIdx.x >> 5) * NR_WIDE_LEARN_WORDS;
        W.M = P.mlp;
        W.scratch = ls;
        W.y = reinterpret_cast<float *>(ls + NR_MLP_WARP_WORDS);
    }
    const int w4 = W4 ? W4 : g.w4;
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned long long gw = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + warp;
    const unsigned long long TW = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long cap = P.capacity;
    // LANES: the lane's mask, level and queue columns, and its sums
    uint32_t *lmc = nullptr;
    unsigned char *ldq = nullptr;
    NrWideLaneAcc LA;
    if constexpr (LANES) {
        unsigned char *lb = smem + nr_wide_block_shm(g, (int)(blockDim.x >> 5)) +
                            (size_t)warp * nr_wide_lane_shm(g.n, W4);
        lmc = reinterpret_cast<uint32_t *>(lb) + lane;
        ldq = lb + (size_t)4 * W4 * 32 * 4 + lane;
        nr_wide_lane_acc_zero(LA);
    }
    __shared__ NrWideAcc s_acc[NR_WIDE_BLOCK / 32];          // as in nr_grid_wide_kernel
    NrWideAcc &A = s_acc[warp];
    if (lane == 0) nr_wide_acc_init(A);
    if (P.resume && blockIdx.x == 0 && threadIdx.x == 0) {
        A.R = P.init_R; A.et = P.init_et; A.es = P.init_es; A.net = P.init_net;
        A.nodes = P.init_nodes; A.leaves = P.init_leaves; A.dead = P.init_dead; A.trunc = P.init_trunc;
        A.spilled = P.init_spilled;
    }
    __syncwarp();
    NrWideOut O;
    O.mask = P.mask;
    O.mass = P.mass;
    O.key = P.key;
    O.count = P.top;
    O.cap = cap;
    O.shift = P.shift;
    O.nb = P.nb;
    O.hist = s_hist;
    int stop = 0, wave = 0;
    unsigned long long live = 0;
    for (; wave < P.max_waves; ++wave) {
        int bsel;
        nr_bucket_select(P.bcount, P.nb, &bsel, &live);
        if (live == 0) break;                               // queue empty
        stop = nr_wide_stop_test(P.wpart + (size_t)((wave + 1) & 1) * gridDim.x, wave == 0 && !P.resume,
                                 P.target_on, P.target_fix, P.max_nodes);
        if (stop) break;
        // reclaim freed slots once they are a large part of the used arena
        unsigned long long used = min(__ldcg(P.top), cap);
        if (used > live && ((used > cap / 2 && used - live >= used / 4) || used > cap - cap / 8)) {
            if (!nr_bucket_compact<W4>(P, used, live)) break;
            used = live;
        }
        // gather the slots of bucket bsel: the whole bucket is this wave
        unsigned long long *wl = P.wave_len + (wave & 1);
        for (unsigned long long s0 = gw * 32; s0 < used; s0 += TW * 32) {
            const unsigned long long s = s0 + lane;
            const bool hit = s < used && __ldcg(P.key + s) == (unsigned char)bsel;
            const unsigned mk = __ballot_sync(NR_FULL, hit);
            if (!mk) continue;
            unsigned long long base = 0;
            if (lane == 0) base = atomicAdd(wl, (unsigned long long)__popc(mk));
            base = __shfl_sync(NR_FULL, base, 0);
            if (hit) {
                __stcg(P.list + base + __popc(mk & ((1u << lane) - 1u)), (unsigned)s);
                __stcg(P.key + s, (unsigned char)NR_WIDE_FREE);
            }
        }
        for (int b = threadIdx.x; b < P.nb; b += blockDim.x) s_hist[b] = 0u;
        if (!nr_grid_sync(P.bar_count, P.bar_gen, P.status, P.timeout_ns)) break;
        // run the wave; children go to the end of the arena
        const unsigned long long n_in = __ldcg(wl);
        if (threadIdx.x == 0 && blockIdx.x == 0) {
            atomicAdd(P.bcount + bsel, (unsigned long long)0 - n_in);
            P.wave_len[(wave + 1) & 1] = 0;
            if (n_in > P.stats[0]) P.stats[0] = n_in;
        }
        // LANES: a wave of at least lane_min_wave records takes one lane a record; a smaller one
        // the whole warp a record (a lane's search is a long serial chain: in a wave that leaves
        // most lanes idle the warp's parallel search ends sooner)
        bool lane_wave = false;
        if constexpr (LANES) lane_wave = n_in >= P.lane_min_wave;
        if (lane_wave) {
            if constexpr (LANES) {
                for (unsigned long long b0 = gw * 32; b0 < n_in; b0 += TW * 32) {
                    const unsigned long long idx = b0 + lane;
                    const bool valid = idx < n_in;
                    double mass = 0.0;
                    if (valid) {
                        const unsigned long long s = __ldcg(P.list + idx);
#pragma unroll
                        for (int k = 0; k < W4; ++k) {
                            const uint4 q = __ldcg(P.mask + s * W4 + k);
                            lmc[32 * (4 * k)] = q.x; lmc[32 * (4 * k + 1)] = q.y;
                            lmc[32 * (4 * k + 2)] = q.z; lmc[32 * (4 * k + 3)] = q.w;
                        }
                        mass = __ldcg(P.mass + s);
                    }
                    nr_wide_lane_step<W4>(g, v, lmc, ldq, valid, mass, P.eps, O, LA, P.status);
                    __syncwarp();
                }
                nr_wide_lane_fold(LA, A);
            }
        } else {
            for (unsigned long long idx = gw; idx < n_in; idx += TW) {
                const unsigned long long s = __ldcg(P.list + idx);
                nr_wide_load_mask(v.m, P.mask + s * w4, w4);
                const double mass = __ldcg(P.mass + s);
                __syncwarp();
                nr_wide_step<W4>(g, v, mass, P.eps, O, A, P.fork != 0, P.border, LEARN ? &W : nullptr);
            }
        }
        __syncthreads();
        for (int b = threadIdx.x; b < P.nb; b += blockDim.x)
            if (s_hist[b]) atomicAdd(P.bcount + b, (unsigned long long)s_hist[b]);
        nr_wide_write_share(P.wpart + (size_t)(wave & 1) * gridDim.x, A);
        if (!nr_grid_sync(P.bar_count, P.bar_gen, P.status, P.timeout_ns)) break;
    }
    if (threadIdx.x == 0 && blockIdx.x == 0) {
        if (wave == P.max_waves) atomicOr(P.status, NR_DEV_ERR_WAVES);
        P.stop_info[0] = wave;
        P.stop_info[1] = stop;
        P.stats[1] = live;
    }
    nr_wide_block_partial(P.partials + blockIdx.x, A);
}
