// nr_lane.cuh -- warp-per-instance engine with one lane per subproblem, for
// undirected simple graphs of up to 16 nodes.
//
// nr_warp_kernel spreads one subproblem over a lane group (a lane per node:
// ballot BFS, shuffled path walk), so a warp expands two subproblems of a K15
// instance at a time and a whole step costs ~700 warp instructions per
// subproblem.  Here each lane expands its own subproblem with bit operations
// on 16-bit adjacency rows, so one step takes a page of up to 32 records and
// a breadth-first wave of <= 32 records is a single step:
//   * a record carries the subproblem's not-down rows (16 rows of 16 bits) next
//     to its mask and mass; a child's rows are its parent's less its down edge,
//     so no row is ever rebuilt from the mask;
//   * BFS per lane: frontier sets as bit masks, the next level is the union of
//     the frontier's rows; dst is tested against the frontier first, so the
//     level that reaches dst is never expanded;
//   * the same parent rule as the lane-group engine (the smallest frontier node
//     adjacent to a node discovers it), hence the same path and the same
//     children (workingPad/main.cu:114-283), and the same FP64 products;
//   * with one bucket (breadth-first waves, exhaustive pages) a warp-wide prefix
//     over the lanes' child counts places every child of a step with one page
//     allocation; with mass buckets, children are pushed one hop index at a
//     time with warp-aggregated allocation per bucket;
//   * the root's rows come from the topology's table when no edge is certainly
//     down (the usual case), so an instance starts without a gather.
// The queue (bucket chains, free-page stack, wave and page modes, spills and
// hand-over) is the one nr_warp.cuh describes; a popped page is returned to the
// free stack as soon as its records are loaded, so its step's children can
// reuse it.
#pragma once

#include "nr_warp.cuh"

#define NR_LANE_MAX_N 16
#define NR_LANE_MAX_W4 2        // a simple graph on <= 16 nodes has <= 120 edges: 8 mask words
#define NR_LANE_ROW_WORDS 8     // 16 rows of 16 bits, two to a word
#define NR_LANE_STEP_CAP (1ll << 26)   // steps (pages) per instance: 2^31 subproblems
#define NR_LANE_STATUS_CHECK NR_WARP_STATUS_CHECK

// A path hop in a lane kernel's hop column.  Rows of RB bits (RB = 16: graphs of <= 16 nodes,
// <= 120 edges; RB = 32: <= 32 nodes, <= 496 edges): edge id (EB bits), its nodes u and x (NB
// bits each), and above bit KS a p-ordered branch order's sort key (16 or 13 bits).
template <int RB> struct NrHop;
template <> struct NrHop<16> { static constexpr int EB = 7, NB = 4, KS = 16; };
template <> struct NrHop<32> { static constexpr int EB = 9, NB = 5, KS = 19; };
template <int RB> __device__ __forceinline__ int nr_hop_e(uint32_t h) { return (int)(h & ((1u << NrHop<RB>::EB) - 1u)); }
template <int RB> __device__ __forceinline__ int nr_hop_u(uint32_t h)
{
    return (int)((h >> NrHop<RB>::EB) & ((1u << NrHop<RB>::NB) - 1u));
}
template <int RB> __device__ __forceinline__ int nr_hop_x(uint32_t h)
{
    return (int)((h >> (NrHop<RB>::EB + NrHop<RB>::NB)) & ((1u << NrHop<RB>::NB) - 1u));
}
template <int RB> __device__ __forceinline__ uint32_t nr_hop_make(uint32_t e, uint32_t u, uint32_t x)
{
    return e | (u << NrHop<RB>::EB) | (x << (NrHop<RB>::EB + NrHop<RB>::NB));
}
#define NR_HOP_E(h) nr_hop_e<16>(h)
#define NR_HOP_U(h) nr_hop_u<16>(h)
#define NR_HOP_X(h) nr_hop_x<16>(h)
// row words of a lane's rows: 16-bit rows two to a word, 32-bit rows one a word
template <int RB> __host__ __device__ constexpr int nr_lane_rw() { return RB == 16 ? 8 : 32; }

// shared memory of one warp
__host__ __device__ inline size_t nr_lane_shm_bytes(int n_buckets, int pages)
{
    size_t b = 32 * sizeof(NrLaneAcc);                       // per-lane sums and counters
    b += (size_t)NR_LANE_ROW_WORDS * 32 * 4;                 // each lane's rows, [word][lane]
    b += (size_t)NR_LANE_MAX_N * 32 * 4;                     // BFS frontiers, then path hops, [level][lane]
    b += (size_t)n_buckets * 2;
    b = (b + 3) & ~size_t(3);
    b += (size_t)(n_buckets / 32) * 4;
    b += (size_t)pages * 2;
    b += (size_t)pages;
    b = (b + 1) & ~size_t(1);
    b += (size_t)pages * 2;
    return (b + 15) & ~size_t(15);
}

// row of node u (its not-down neighbours) from the lane's rows in shared memory
template <int RB = 16>
__device__ __forceinline__ uint32_t nr_lane_row(const uint32_t *my_rows, int u)
{
    if constexpr (RB == 16) return (my_rows[(u >> 1) * 32] >> ((u & 1) << 4)) & 0xffffu;
    else return my_rows[u * 32];
}

template <int N>
__device__ __forceinline__ uint32_t nr_pick(const uint32_t (&a)[N], int i)
{
    uint32_t r = a[0];
#pragma unroll
    for (int k = 1; k < N; ++k)
        if (k == i) r = a[k];
    return r;
}

// The root record of an instance, at slot 0 of page rpg (all lanes): the mask from p (p <= 0
// down, p >= 1 up, else unknown, main.cu:717-748; 16 edges a word, each half-warp ORs one word
// together), the rows (rows 2k and 2k+1 share word k: the topology's table when no edge is
// certainly down, else lane u gathers its not-down neighbours), mass 1.
template <int W4>
__device__ __forceinline__ void nr_lane_root(const NrSmallGraph &g, const unsigned char *gb, const unsigned char *gs,
                                             uint4 *sl_mask, uint4 *sl_rows, double *sl_mass, int rpg)
{
    constexpr int RW = NR_LANE_ROW_WORDS;
    const int lane = threadIdx.x & 31;
    const double *pt = reinterpret_cast<const double *>(gb + g.off_p);
    uint32_t *rw = reinterpret_cast<uint32_t *>(sl_mask + (size_t)rpg * NR_PAGE * W4);
    bool down = false;
#pragma unroll
    for (int e0 = 0; e0 < 64 * W4; e0 += 32) {
        const int e = e0 + lane;
        uint32_t v = 0u;
        if (e < g.e) {
            const double pe = pt[e];
            down = down || pe <= 0.0;
            v = (uint32_t)((pe <= 0.0) ? NR_EDGE_DOWN : (pe >= 1.0) ? NR_EDGE_UP : NR_EDGE_UNKNOWN)
                << ((e & 15) << 1);
        }
        v |= __shfl_xor_sync(NR_FULL, v, 8);
        v |= __shfl_xor_sync(NR_FULL, v, 4);
        v |= __shfl_xor_sync(NR_FULL, v, 2);
        v |= __shfl_xor_sync(NR_FULL, v, 1);
        if ((lane & 15) == 0) rw[(e0 >> 4) + (lane >> 4)] = v;
    }
    uint32_t *rr = reinterpret_cast<uint32_t *>(sl_rows + (size_t)rpg * NR_PAGE * (RW / 4));
    if (!__any_sync(NR_FULL, down)) {
        if (lane < RW) rr[lane] = reinterpret_cast<const uint32_t *>(gs + g.off_root_rows)[lane];
    } else {
        const int *start = reinterpret_cast<const int *>(gs + g.off_start);
        const uint32_t *list = reinterpret_cast<const uint32_t *>(gs + g.off_list);
        uint32_t r = 0;
        if (lane < g.n)
            for (int j = start[lane]; j < start[lane + 1]; ++j) {
                const uint32_t a = list[j];
                if (pt[a >> 8] > 0.0) r |= 1u << (a & 31u);
            }
        const uint32_t hi = __shfl_down_sync(NR_FULL, r, 1);
        if (lane < 2 * RW && !(lane & 1)) rr[lane >> 1] = r | (hi << 16);
    }
    if (lane == 0) sl_mass[(size_t)rpg * NR_PAGE] = 1.0;
}

// One lane's path: BFS from src over the not-down rows (the frontier of level l goes to
// my_hop[l]; dst is tested against the frontier first, so the level that reaches it is never
// expanded), then the walk dst -> src (the parent of a node on level l+1 is the smallest node
// of frontier l adjacent to it; hop l = (u, x) with its edge id replaces frontier l).  Returns
// the hops L (0 for a dead end or an inactive lane); live = dst reached; nch = the UNKNOWN hops,
// i.e. the lane's children; bad = a failed internal check (2 levels, 3 parent, 4 edge id).
template <int NW, int RB = 16>
__device__ __forceinline__ int nr_lane_path(const uint32_t *my_rows, uint32_t *my_hop, const uint32_t (&wc)[NW],
                                            const uint16_t *eid, int n, int ge, int src, int dst, bool active,
                                            bool &live, int &nch, int &bad)
{
    const int es = n <= 8 ? 8 : n <= 16 ? 16 : 32;  // edge-id table stride (the host's group width)
    int L = 0;
    live = false;
    nch = 0;
    bad = 0;
    if (!active) return 0;
    if (src == dst) { live = true; return 0; }
    const uint32_t rd = nr_lane_row<RB>(my_rows, dst);
    uint32_t F = 1u << src, vis = F;
    for (;;) {                                      // every level adds a node: at most n - 1 levels
        if (L >= RB) { bad = 2; return 0; }
        my_hop[32 * L] = F;
        if (rd & F) { ++L; live = true; break; }    // dst is on the next level
        uint32_t nf = 0u;
        for (uint32_t t = F; t; t &= t - 1u) nf |= nr_lane_row<RB>(my_rows, __ffs(t) - 1);
        nf &= ~vis;
        if (!nf) return 0;                          // a dead end has no path: no hops, no children
        vis |= nf;
        F = nf;
        ++L;
    }
    int x = dst;
    for (int l = L - 1; l >= 0; --l) {
        const int u = __ffs(nr_lane_row<RB>(my_rows, x) & my_hop[32 * l]) - 1;
        if (u < 0 || u >= n) { bad = 3; return 0; }
        const uint32_t e = eid[u * es + x];
        if ((int)e >= ge || e >= (1u << NrHop<RB>::EB)) { bad = 4; return 0; }
        my_hop[32 * l] = nr_hop_make<RB>(e, (uint32_t)u, (uint32_t)x);
        nch += ((nr_pick(wc, (int)e >> 4) >> ((e & 15) << 1)) & 3u) == 3u;
        x = u;
    }
    return L;
}

// A sort key non-decreasing in p, in the hop word's key bits (16 or 13): the top bits of p's bit
// pattern (positive doubles order as their bit patterns do), saturated; p <= 0 gives 0.  Equal
// keys compare p itself.
template <int RB = 16>
__device__ __forceinline__ uint32_t nr_p_key(double p)
{
    constexpr int KB = 32 - NrHop<RB>::KS;
    const long long b = __double_as_longlong(p);
    return b <= 0 ? 0u : (uint32_t)min((unsigned long long)b >> (54 - KB), (1ull << KB) - 1ull);
}

// Branch order of one lane's path hops my_hop[32 l], l = 0..L-1 src side first: dst side
// first (reversed), or by p (ascending / descending, stable in path order -- the oracle's
// insertion sort of the src -> dst path).  Known hops move too but make no child, so only
// the UNKNOWN hops' relative order matters.  The sort keys ride in the hop words' top bits.
template <int RB = 16>
__device__ __forceinline__ void nr_lane_branch_order(uint32_t *my_hop, int L, int border, const double *pt)
{
    constexpr int KS = NrHop<RB>::KS;
    if (border == NR_BORDER_DST) {
        for (int i = 0, j = L - 1; i < j; ++i, --j) {
            const uint32_t t = my_hop[32 * i];
            my_hop[32 * i] = my_hop[32 * j];
            my_hop[32 * j] = t;
        }
        return;
    }
    const bool desc = (border == NR_BORDER_P_DESC);
    for (int i = 0; i < L; ++i) {
        const uint32_t h = my_hop[32 * i];
        my_hop[32 * i] = (h & ((1u << KS) - 1u)) | (nr_p_key<RB>(pt[nr_hop_e<RB>(h)]) << KS);
    }
    for (int i = 1; i < L; ++i) {
        const uint32_t hp = my_hop[32 * i];
        const uint32_t ke = hp >> KS;
        int j = i - 1;
        while (j >= 0) {
            const uint32_t hj = my_hop[32 * j];
            const uint32_t kj = hj >> KS;
            bool after = desc ? kj < ke : kj > ke;          // j moves past i: strictly out of order
            if (kj == ke) {
                const double pj = pt[nr_hop_e<RB>(hj)], pe = pt[nr_hop_e<RB>(hp)];
                after = desc ? pj < pe : pj > pe;
            }
            if (!after) break;
            my_hop[32 * (j + 1)] = hj;
            --j;
        }
        my_hop[32 * (j + 1)] = hp;
    }
}

// Child record at slot s: the parent's mask blocks, then the one word that differs (hop edge e
// down; this thread's later store to the same address wins); the parent's rows less the down
// edge cu - cv; mass cm.  wv = the parent's (current) mask word of e.  32-bit rows
// (nr_lane_write_child32) are copied from the lane's shared-memory column, not registers.
template <int W4>
__device__ __forceinline__ void nr_lane_write_child32(uint4 *sl_mask, uint4 *sl_rows, double *sl_mass, int s,
                                                      const uint32_t (&wc)[4 * W4], const uint32_t *my_rows, int e,
                                                      uint32_t wv, int cu, int cv, double cm)
{
    uint4 *d = sl_mask + (size_t)s * W4;
#pragma unroll
    for (int kk = 0; kk < W4; ++kk)
        d[kk] = make_uint4(wc[4 * kk], wc[4 * kk + 1], wc[4 * kk + 2], wc[4 * kk + 3]);
    reinterpret_cast<uint32_t *>(d)[e >> 4] = wv & ~(3u << ((e & 15) << 1));
    uint4 *dr = sl_rows + (size_t)s * 8;
#pragma unroll
    for (int kk = 0; kk < 8; ++kk) {
        uint32_t r[4];
#pragma unroll
        for (int i = 0; i < 4; ++i) {
            const int u = 4 * kk + i;
            r[i] = my_rows[32 * u] & ~(u == cu ? 1u << cv : 0u) & ~(u == cv ? 1u << cu : 0u);
        }
        dr[kk] = make_uint4(r[0], r[1], r[2], r[3]);
    }
    sl_mass[s] = cm;
}

template <int W4>
__device__ __forceinline__ void nr_lane_write_child(uint4 *sl_mask, uint4 *sl_rows, double *sl_mass, int s,
                                                    const uint32_t (&wc)[4 * W4],
                                                    const uint32_t (&rw)[NR_LANE_ROW_WORDS],
                                                    const uint32_t *my_rows, int e, uint32_t wv, int cu, int cv,
                                                    double cm)
{
    constexpr int RW = NR_LANE_ROW_WORDS;
    uint4 *d = sl_mask + (size_t)s * W4;
#pragma unroll
    for (int kk = 0; kk < W4; ++kk)
        d[kk] = make_uint4(wc[4 * kk], wc[4 * kk + 1], wc[4 * kk + 2], wc[4 * kk + 3]);
    reinterpret_cast<uint32_t *>(d)[e >> 4] = wv & ~(3u << ((e & 15) << 1));
    const int wu = cu >> 1, wv2 = cv >> 1;
    const uint32_t bu = 1u << (cv + ((cu & 1) << 4));
    const uint32_t bv = 1u << (cu + ((cv & 1) << 4));
    uint4 *dr = sl_rows + (size_t)s * (RW / 4);
#pragma unroll
    for (int kk = 0; kk < RW / 4; ++kk)
        dr[kk] = make_uint4(rw[4 * kk], rw[4 * kk + 1], rw[4 * kk + 2], rw[4 * kk + 3]);
    uint32_t *drw = reinterpret_cast<uint32_t *>(dr);
    if (wu == wv2) {
        drw[wu] = my_rows[32 * wu] & ~(bu | bv);
    } else {
        drw[wu] = my_rows[32 * wu] & ~bu;
        drw[wv2] = my_rows[32 * wv2] & ~bv;
    }
    sl_mass[s] = cm;
}

template <int W4>
__global__ void __launch_bounds__(NR_WARP_BLOCK_MAX, 2) nr_lane_kernel(NrWarpParams P)
{
    constexpr int NW = 4 * W4;
    constexpr int RW = NR_LANE_ROW_WORDS;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const unsigned lt_mask = (1u << lane) - 1u;
    const int NB = P.n_buckets, NP = P.pages;

    NrWarpShm sh;
    NrLaneAcc *acc_base;
    uint32_t *my_rows, *my_hop;
    {
        unsigned char *b = smem + (size_t)warp * nr_lane_shm_bytes(NB, NP);
        acc_base = reinterpret_cast<NrLaneAcc *>(b);
        b += 32 * sizeof(NrLaneAcc);
        my_rows = reinterpret_cast<uint32_t *>(b) + lane;          // word k at my_rows[32 k]
        b += (size_t)RW * 32 * 4;
        my_hop = reinterpret_cast<uint32_t *>(b) + lane;           // level l at my_hop[32 l]
        b += (size_t)NR_LANE_MAX_N * 32 * 4;
        size_t o = 0;
        sh.masks = nullptr;
        sh.heads = reinterpret_cast<short *>(b + o); o += (size_t)NB * 2; o = (o + 3) & ~size_t(3);
        sh.bitmap = reinterpret_cast<uint32_t *>(b + o); o += (size_t)(NB / 32) * 4;
        sh.pnext = reinterpret_cast<short *>(b + o); o += (size_t)NP * 2;
        sh.pcnt = b + o; o += (size_t)NP; o = (o + 1) & ~size_t(1);
        sh.freel = reinterpret_cast<short *>(b + o);
    }
    const size_t gw = (size_t)blockIdx.x * (blockDim.x >> 5) + warp;
    uint4 *sl_mask = P.slab_mask + gw * (size_t)NP * NR_PAGE * W4;
    double *sl_mass = P.slab_mass + gw * (size_t)NP * NR_PAGE;
    uint4 *sl_rows = reinterpret_cast<uint4 *>(P.slab_rows) + gw * (size_t)NP * NR_PAGE * (RW / 4);
    const bool use_eps = P.eps > 0.0;
    const long long step_cap = P.step_cap > 0 ? P.step_cap : NR_LANE_STEP_CAP;

    for (;;) {
        int ii = 0;
        if (lane == 0) ii = atomicAdd(P.next_inst, 1);
        ii = __shfl_sync(NR_FULL, ii, 0);
        if (ii >= P.n_inst) break;
        const NrSmallGraph g = P.inst[ii];
        const unsigned char *gb = P.blob + g.blob_off;
        const unsigned char *gs = P.blob + g.struct_off;
        const double *pt = reinterpret_cast<const double *>(gb + g.off_p);
        const uint16_t *eid = reinterpret_cast<const uint16_t *>(gs + g.off_eid);
        const int n = g.n, src = g.src, dst = g.dst;
        const long long t0 = nr_globaltimer();

        // reset the private queue; the root is the only subproblem
        for (int b = lane; b < NB; b += 32) sh.heads[b] = -1;
        for (int b = lane; b < NB / 32; b += 32) sh.bitmap[b] = 0u;
        for (int p = lane; p < NP; p += 32) { sh.freel[p] = (short)(NP - 1 - p); sh.pnext[p] = -1; sh.pcnt[p] = 0; }
        int top = NP;
        __syncwarp();
        int rpg = 0;
        if (lane == 0) {
            const int rb = nr_bucket(1.0, P.shift, NB);
            rpg = sh.freel[--top];
            sh.heads[rb] = (short)rpg;
            sh.pcnt[rpg] = 1;
            sh.pnext[rpg] = -1;
            sh.bitmap[rb >> 5] |= 1u << (rb & 31);
        }
        top = __shfl_sync(NR_FULL, top, 0);
        rpg = __shfl_sync(NR_FULL, rpg, 0);
        nr_lane_root<W4>(g, gb, gs, sl_mask, sl_rows, sl_mass, rpg);
        __syncwarp();

        NrLaneAcc &acc = acc_base[lane];
        nr_acc_zero(acc);
        // queued mass and count.  Mass buckets: this lane's pushes - pops.  One bucket: every
        // queued record is on bucket 0's chain, so the stop test sums that chain instead
        // (lane i takes record i of each page) and pushes and pops keep no account.
        const bool one_bucket = P.shift < 0;
        int check = 0;                          // which internal check failed (0: none)
        NrFix qacc = (lane == 0 && !one_bucket) ? nr_fix_of(1.0) : nr_fix_zero();
        long long qcount = (lane == 0 && !one_bucket) ? 1 : 0;
        auto chain_sum = [&]() {
            if (!one_bucket) return;
            qacc = nr_fix_zero();
            qcount = 0;
            int pg = sh.heads[0];
            for (int k = 0; pg >= 0 && k < NP; pg = sh.pnext[pg], ++k)   // a chain holds <= NP pages
                if (lane < (int)sh.pcnt[pg]) {
                    nr_fix_add_mass(qacc, sl_mass[(size_t)pg * NR_PAGE + lane]);
                    qcount++;
                }
            if (pg >= 0) check = 6;                  // longer than the pool: the chain is corrupt
        };
        int waves = 0, status = 0;
        unsigned long long max_wave = 0;
        bool abandon = false;
        long long steps = 0;

        for (;;) {
            // fullest (lowest-index) non-empty bucket; an empty queue ends the run before the other
            // tests, as in the oracle's wave loop (pathdecomp.c: empty, target width, budget)
            const uint32_t wbm = (lane < NB / 32) ? sh.bitmap[lane] : 0u;
            const unsigned nz = __ballot_sync(NR_FULL, wbm != 0u);
            if (!nz) break;
            if (P.wave_mode && P.target > 0.0) {     // exact: ESP + queued mass <= target
                chain_sum();
                if (check) { status = NR_LANE_STATUS_CHECK; max_wave = (unsigned long long)check; break; }
                NrFix w = qacc;
                nr_fix_add(w, acc.et);
                nr_fix_add(w, acc.es);
                w = nr_fix_warp_sum(w);
                if (nr_fix_le(w, P.target_fix)) { status = 1; break; }
            }
            if (P.max_nodes && nr_warp_sum_u64(acc.nodes) >= P.max_nodes) {
                if (P.wave_mode) { status = 3; } else { status = 2; abandon = true; }
                break;
            }
            const int wi = __ffs(nz) - 1;
            const int bk = wi * 32 + __ffs(__shfl_sync(NR_FULL, wbm, wi)) - 1;
            int chain = 0;
            if (lane == 0) {
                chain = sh.heads[bk];
                if (P.wave_mode) {
                    sh.heads[bk] = -1;
                    sh.bitmap[bk >> 5] &= ~(1u << (bk & 31));
                } else {
                    const int nx = sh.pnext[chain];
                    sh.heads[bk] = (short)nx;
                    sh.pnext[chain] = -1;
                    if (nx < 0) sh.bitmap[bk >> 5] &= ~(1u << (bk & 31));
                }
            }
            chain = __shfl_sync(NR_FULL, chain, 0);
            __syncwarp();
            ++waves;
            unsigned long long wave_items = 0;
            for (int pg = chain; pg >= 0 && !abandon;) {
                const int cnt = sh.pcnt[pg];
                const int nxt = sh.pnext[pg];
                wave_items += cnt;
                // one step: lane i expands record i of the page
                if (++steps > step_cap) { check = 1; abandon = true; break; }
                const bool valid = lane < cnt;
                const size_t slot = (size_t)pg * NR_PAGE + lane;
                uint32_t wc[NW], rw[RW];
                double mass = 0.0;
                if (valid) {
#pragma unroll
                    for (int k = 0; k < W4; ++k) {
                        const uint4 q = sl_mask[slot * W4 + k];
                        wc[4 * k] = q.x; wc[4 * k + 1] = q.y; wc[4 * k + 2] = q.z; wc[4 * k + 3] = q.w;
                    }
#pragma unroll
                    for (int k = 0; k < RW / 4; ++k) {
                        const uint4 q = sl_rows[slot * (RW / 4) + k];
                        rw[4 * k] = q.x; rw[4 * k + 1] = q.y; rw[4 * k + 2] = q.z; rw[4 * k + 3] = q.w;
                    }
                    mass = sl_mass[slot];
                } else {
#pragma unroll
                    for (int k = 0; k < NW; ++k) wc[k] = 0u;
#pragma unroll
                    for (int k = 0; k < RW; ++k) rw[k] = 0u;
                }
#pragma unroll
                for (int k = 0; k < RW; ++k) my_rows[32 * k] = rw[k];
                __syncwarp();                       // every lane holds its record: the page is free
                if (lane == 0) sh.freel[top++] = (short)pg;
                top = __shfl_sync(NR_FULL, top, 0);
                __syncwarp();

                bool active = valid;
                if (valid) {
                    acc.nodes++;
                    if (!one_bucket) {
                        nr_fix_sub(qacc, nr_fix_of(mass));
                        qcount--;
                    }
                    if (use_eps && mass < P.eps) {         // main.cu:537-543
                        acc.trunc++;
                        nr_fix_add_mass(acc.et, mass);
                        active = false;
                    }
                }

                bool live;
                int nch, bad;
                const int L = nr_lane_path(my_rows, my_hop, wc, eid, n, g.e, src, dst, active, live, nch, bad);
                if (P.border != NR_BORDER_SRC && L > 1) nr_lane_branch_order(my_hop, L, P.border, pt);
                if (active && !live && !bad) acc.dead++;

                {
                    const unsigned bm = __ballot_sync(NR_FULL, bad != 0);
                    if (bm) {                       // record the first failing lane's check and stop
                        check = __shfl_sync(NR_FULL, bad, __ffs(bm) - 1);
                        abandon = true;
                        break;
                    }
                }
                // the path src side first: child h = earlier UNKNOWN hops up, hop h down;
                // FP64 masses in path order, as the lane-group engine and the oracle
                double Pm = mass;
                if (P.shift < 0) {
                    // one bucket: every child of the step goes to the same chain, so one warp-wide
                    // prefix over the lanes' child counts places them all (the head page's free
                    // slots first, then fresh pages from the free stack)
                    int pre = nch;
#pragma unroll
                    for (int off = 1; off < 32; off <<= 1) {
                        const int t = __shfl_up_sync(NR_FULL, pre, off);
                        if (lane >= off) pre += t;
                    }
                    const int total = __shfl_sync(NR_FULL, pre, 31);
                    pre -= nch;
                    int hA = -1, cA = 0, nA = 0, npg = 0;
                    const int top0 = top;
                    if (lane == 0 && total > 0) {
                        const int hd = sh.heads[0];
                        const int c = (hd >= 0) ? sh.pcnt[hd] : NR_PAGE;
                        nA = min(total, NR_PAGE - c);
                        if (nA > 0) { hA = hd; cA = c; sh.pcnt[hd] = (unsigned char)(c + nA); }
                        const int rest = total - nA;
                        npg = min((rest + NR_PAGE - 1) / NR_PAGE, top0);
                        int prev = hd;
                        for (int i = 0; i < npg; ++i) {       // fresh pages, the last one the new head
                            const int pgi = sh.freel[top0 - 1 - i];
                            sh.pnext[pgi] = (short)prev;
                            sh.pcnt[pgi] = (unsigned char)min(NR_PAGE, rest - NR_PAGE * i);
                            prev = pgi;
                        }
                        if (npg > 0) {
                            sh.heads[0] = (short)prev;
                            sh.bitmap[0] |= 1u;
                        }
                    }
                    hA = __shfl_sync(NR_FULL, hA, 0);
                    cA = __shfl_sync(NR_FULL, cA, 0);
                    nA = __shfl_sync(NR_FULL, nA, 0);
                    npg = __shfl_sync(NR_FULL, npg, 0);
                    top = top0 - npg;
                    __syncwarp();
                    int q = pre;                            // this lane's next child index
                    for (int h = 0; h < L; ++h) {
                        const uint32_t hp = my_hop[32 * h];
                        const int e = NR_HOP_E(hp);
                        const int ew = e >> 4;
                        const uint32_t wv = nr_pick(wc, ew);
                        if (((wv >> ((e & 15) << 1)) & 3u) != 3u) continue;
                        const int cu = NR_HOP_U(hp), cv = NR_HOP_X(hp);
                        const double pe = pt[e];
                        const double cm = __dmul_rn(Pm, __dsub_rn(1.0, pe));
                        Pm = __dmul_rn(Pm, pe);
                        int s = -1;
                        if (q < nA) {
                            s = hA * NR_PAGE + cA + q;
                        } else {
                            const int r = q - nA;
                            if ((r >> 5) < npg) s = sh.freel[top0 - 1 - (r >> 5)] * NR_PAGE + (r & 31);
                        }
                        ++q;
                        if (s >= 0) {
                            nr_lane_write_child<W4>(sl_mask, sl_rows, sl_mass, s, wc, rw, my_rows, e, wv, cu, cv, cm);
                        } else if (P.escalate) {
                            abandon = true;
                        } else {                          // queue full: mass to ESP (main.cu:245-252)
                            acc.spilled++;
                            nr_fix_add_mass(acc.es, cm);
                        }
#pragma unroll
                        for (int kk = 0; kk < NW; ++kk)   // later children see hop h up
                            if (kk == ew) wc[kk] &= ~(2u << ((e & 15) << 1));
                    }
                    abandon = __any_sync(NR_FULL, abandon);
                }
                const int Lmax = (P.shift < 0) ? 0 : (int)__reduce_max_sync(NR_FULL, (unsigned)L);
                for (int h = 0; h < Lmax; ++h) {
                    bool has_child = false;
                    double cm = 0.0;
                    int e = 0, cu = 0, cv = 0;
                    uint32_t wv = 0u;
                    if (h < L) {
                        const uint32_t hp = my_hop[32 * h];
                        e = NR_HOP_E(hp);
                        cu = NR_HOP_U(hp);
                        cv = NR_HOP_X(hp);
                        wv = nr_pick(wc, e >> 4);
                        if (((wv >> ((e & 15) << 1)) & 3u) == 3u) {
                            const double pe = pt[e];
                            cm = __dmul_rn(Pm, __dsub_rn(1.0, pe));
                            Pm = __dmul_rn(Pm, pe);
                            has_child = true;
                        }
                    }
                    const bool was_unknown = has_child;
                    const int cb = has_child ? nr_bucket(cm, P.shift, NB) : 0;
                    unsigned pend = __ballot_sync(NR_FULL, has_child);
                    while (pend) {
                        const int bsel = __shfl_sync(NR_FULL, cb, __ffs(pend) - 1);
                        const unsigned m = __ballot_sync(NR_FULL, has_child && cb == bsel);
                        const int nm = __popc(m);
                        int hA = -1, cA = 0, nA = 0, hB = -1;
                        if (lane == 0) {
                            const int hd = sh.heads[bsel];
                            const int c = (hd >= 0) ? sh.pcnt[hd] : NR_PAGE;
                            nA = min(nm, NR_PAGE - c);
                            if (nA > 0) { hA = hd; cA = c; sh.pcnt[hd] = (unsigned char)(c + nA); }
                            const int rest = nm - nA;
                            if (rest > 0 && top > 0) {
                                hB = sh.freel[--top];
                                sh.pnext[hB] = (short)hd;
                                sh.pcnt[hB] = (unsigned char)rest;
                                sh.heads[bsel] = (short)hB;
                                sh.bitmap[bsel >> 5] |= 1u << (bsel & 31);
                            }
                        }
                        top = __shfl_sync(NR_FULL, top, 0);
                        hA = __shfl_sync(NR_FULL, hA, 0);
                        cA = __shfl_sync(NR_FULL, cA, 0);
                        nA = __shfl_sync(NR_FULL, nA, 0);
                        hB = __shfl_sync(NR_FULL, hB, 0);
                        __syncwarp();
                        if (has_child && cb == bsel) {
                            const int r = __popc(m & lt_mask);
                            const int s = (r < nA) ? hA * NR_PAGE + cA + r : (hB >= 0 ? hB * NR_PAGE + (r - nA) : -1);
                            if (s >= 0) {
                                nr_lane_write_child<W4>(sl_mask, sl_rows, sl_mass, s, wc, rw, my_rows, e, wv, cu, cv, cm);
                                nr_fix_add_mass(qacc, cm);
                                qcount++;
                            } else if (P.escalate) {
                                abandon = true;
                            } else {                      // queue full: mass to ESP (main.cu:245-252)
                                acc.spilled++;
                                nr_fix_add_mass(acc.es, cm);
                            }
                            has_child = false;
                        }
                        pend = __ballot_sync(NR_FULL, has_child);
                    }
                    if (was_unknown) {                    // later children see hop h up
                        const int ew = e >> 4;
                        const uint32_t ubit = 2u << ((e & 15) << 1);
#pragma unroll
                        for (int k = 0; k < NW; ++k)
                            if (k == ew) wc[k] &= ~ubit;
                    }
                    abandon = __any_sync(NR_FULL, abandon);
                    if (abandon) break;
                }
                if (live && !abandon) {
                    acc.leaves++;
                    nr_fix_add_mass(acc.R, Pm);
                }
                __syncwarp();                       // my_rows / my_hop are rewritten by the next step
                pg = nxt;
            }
            if (check) { status = NR_LANE_STATUS_CHECK; max_wave = (unsigned long long)check; break; }
            if (abandon) { status = 2; break; }
            if (wave_items > max_wave) max_wave = wave_items;
        }
        const long long t_stop = nr_globaltimer() - t0;
        chain_sum();                                // one bucket: what is left queued
        if (check && status != NR_LANE_STATUS_CHECK) { status = NR_LANE_STATUS_CHECK; max_wave = (unsigned long long)check; }

        const NrFix R = nr_fix_warp_sum(acc.R), et = nr_fix_warp_sum(acc.et), es_ = nr_fix_warp_sum(acc.es);
        const NrFix qm = nr_fix_warp_sum(qacc);
        const unsigned long long nodes = nr_warp_sum_u64(acc.nodes), leaves = nr_warp_sum_u64(acc.leaves);
        const unsigned long long dead = nr_warp_sum_u64(acc.dead), trunc = nr_warp_sum_u64(acc.trunc);
        const unsigned long long spilled = nr_warp_sum_u64(acc.spilled);
        const unsigned long long queued = nr_warp_sum_u64((unsigned long long)qcount);
        if (lane == 0) {
            NrWarpOut o;
            o.R = R; o.et = et; o.es = es_; o.q = qm;
            o.nodes = nodes; o.leaves = leaves; o.dead = dead; o.trunc = trunc; o.spilled = spilled;
            o.queued = queued; o.max_wave = max_wave; o.t_ns = t_stop; o.waves = waves; o.status = status;
            P.out[P.inst_id[ii]] = o;
        }
        __syncwarp();
    }
}
