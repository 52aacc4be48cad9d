// nr_expand.cuh -- the per-subproblem step shared by the engines: optimistic
// BFS over not-down arcs, path extraction, and the disjoint branches of the
// path (child k = first k-1 UNKNOWN path edges up, k-th down; all-up -> R).
//
// Restates workingPad/device_code.cuh:80-194 (bfs_reachable) and
// workingPad/main.cu:114-283 (path_edge_sweep_warp) with a different mapping:
// a warp holds K = 32/G subproblems, G lanes each, lane v of a group owns
// node v.  A node's not-down in-neighbours form one 32-bit row, so one BFS
// level is one AND, one __ballot_sync and one __ffs per lane, and the parent
// of v is the smallest frontier node with a not-down arc to v -- the rule
// the reference kernel follows when one lane scans the frontier bitmask in
// ascending order (device_code.cuh:141-171).  Masses are FP64 products in
// path order (the reference uses float log sums, common.h:60).
#pragma once

#include "nr_device.cuh"

// View of an instance's graph tables (shared or global memory).  The down
// probability of edge e is 1 - p[e], rounded as the host's double subtraction.
struct NrSmemGraph {
    const double *p;
    const uint16_t *eid;      // [G*G] arc (u -> v) -> edge id
    const int *start;         // [n+1] in-arc ranges
    const uint32_t *list;     // in-arcs of v: (eid << 8) | u
};

__device__ __forceinline__ NrSmemGraph nr_smem_graph(const unsigned char *s, const NrSmallGraph &g)
{
    NrSmemGraph v;
    v.p = reinterpret_cast<const double *>(s + g.off_p);
    v.eid = reinterpret_cast<const uint16_t *>(s + g.off_eid);
    v.start = reinterpret_cast<const int *>(s + g.off_start);
    v.list = reinterpret_cast<const uint32_t *>(s + g.off_list);
    return v;
}

struct NrLaneAcc {
    NrFix R, et, es;
    unsigned long long nodes, leaves, dead, trunc, spilled;
};

__device__ __forceinline__ void nr_acc_zero(NrLaneAcc &a)
{
    a.R = a.et = a.es = nr_fix_zero();
    a.nodes = a.leaves = a.dead = a.trunc = a.spilled = 0;
}

// Level-synchronous BFS of every group of the warp over the in-neighbour rows
// `row` (lane v: the nodes u with a usable arc u -> v); one ballot per level.
// Returns whether dst was reached; par = the smallest frontier node with a
// usable arc to v (lane v), level = hops of the shortest path.  All 32 lanes
// call it; groups with search == false take part without searching.
template <int G>
__device__ __forceinline__ bool nr_group_bfs(uint32_t row, bool search, int n, int src, int dst, int &par, int &level)
{
    const int lane = threadIdx.x & 31;
    const int v = lane & (G - 1);
    const int gbase = lane & ~(G - 1);
    uint32_t F = 1u << src, vis = F;
    par = -1;
    level = 0;
    bool found = search && (src == dst);
    bool searching = search && !found;
    while (__any_sync(NR_FULL, searching)) {
        const uint32_t t = row & F;
        const bool hit = searching && (v < n) && (t != 0u) && !((vis >> v) & 1u);
        if (hit) par = __ffs(t) - 1;
        const uint32_t b = __ballot_sync(NR_FULL, hit);
        const uint32_t nf = (G == 32) ? b : ((b >> gbase) & ((1u << G) - 1u));
        if (searching) {
            vis |= nf;
            F = nf;
            ++level;
            if ((vis >> dst) & 1u) { found = true; searching = false; }
            else if (nf == 0u) searching = false;
        }
    }
    return found;
}

// Expand the group's subproblem (mask words in smem at my_m, mass `mass`).
// Every lane of the warp must call this (it uses full-warp shuffles/ballots).
// On return, a lane with has_child holds one child: words w[] and mass cm.
// Leaf mass, dead ends and truncation are accumulated on the group's lane 0.
#define NR_FEAT 16

// Features of the child a lane holds, for the learned scorer (nr_mlp.cuh):
//   0 log2(child mass)/64     1-3 UNKNOWN/up/down edge fractions
//   4 parent path length / n  5 position of the down edge on the path
//   6 p of the down edge      7-9 not-down degree of src, dst, and their min
//                             (a cut-size estimate), over n-1
//   10 log2(parent mass)/64   11 n/64  12 E/512  13-14 zero  15 one
template <int W4>
__device__ __forceinline__ void nr_child_features(float (&f)[NR_FEAT], const uint32_t (&w)[4 * W4], double cm,
                                                  double mass, int L, int h, double pe, int deg_s, int deg_d,
                                                  int n, int E)
{
    int unk = 0, up = 0;
#pragma unroll
    for (int k = 0; k < 4 * W4; ++k) {
        const uint32_t lo = w[k] & 0x55555555u, hi = (w[k] >> 1) & 0x55555555u;
        unk += __popc(lo & hi);
        up += __popc(lo & ~hi);
    }
    const float inv_e = E > 0 ? 1.f / (float)E : 0.f, inv_n1 = n > 1 ? 1.f / (float)(n - 1) : 0.f;
    f[0] = cm > 0.0 ? fmaxf(log2f((float)cm) * (1.f / 64.f), -16.f) : -16.f;   // below FLT_MIN: -16
    f[1] = unk * inv_e;
    f[2] = up * inv_e;
    f[3] = (E - unk - up) * inv_e;
    f[4] = n > 0 ? (float)L / (float)n : 0.f;
    f[5] = L > 0 ? (float)(h + 1) / (float)L : 0.f;
    f[6] = (float)pe;
    f[7] = deg_s * inv_n1;
    f[8] = deg_d * inv_n1;
    f[9] = min(deg_s, deg_d) * inv_n1;
    f[10] = mass > 0.0 ? fmaxf(log2f((float)mass) * (1.f / 64.f), -16.f) : -16.f;
    f[11] = n * (1.f / 64.f);
    f[12] = E * (1.f / 512.f);
    f[13] = 0.f;
    f[14] = 0.f;
    f[15] = 1.f;
}

// Rows carried in the queue records (the warp engine, simple graphs): the
// subproblem's in-neighbour row of node v comes in, and the row used and the
// down edge's endpoints of the lane's child go out, so the child's rows are the
// parent's with that edge's arcs removed.
struct NrRowIO {
    bool have;          // row_in holds node v's not-down in-neighbour row
    uint32_t row_in;
    uint32_t row;       // out: the row used
    int cu, cv;         // out: the lane's child's down hop (cu -> cv)
};

// not-down in-neighbour row of node v from its in-arc list and the mask
__device__ __forceinline__ uint32_t nr_build_row(const NrSmemGraph &sg, const uint32_t *my_m, int v)
{
    uint32_t row = 0;
    const int lo = sg.start[v], hi = sg.start[v + 1];
    int j = lo;
    for (; j + 4 <= hi; j += 4) {          // four independent in-arcs per trip
        const uint32_t a0 = sg.list[j], a1 = sg.list[j + 1], a2 = sg.list[j + 2], a3 = sg.list[j + 3];
        const uint32_t m0 = my_m[a0 >> 12], m1 = my_m[a1 >> 12], m2 = my_m[a2 >> 12], m3 = my_m[a3 >> 12];
        row |= ((m0 >> ((a0 >> 7) & 30u)) & 1u) << (a0 & 31u);
        row |= ((m1 >> ((a1 >> 7) & 30u)) & 1u) << (a1 & 31u);
        row |= ((m2 >> ((a2 >> 7) & 30u)) & 1u) << (a2 & 31u);
        row |= ((m3 >> ((a3 >> 7) & 30u)) & 1u) << (a3 & 31u);
    }
    for (; j < hi; ++j) {
        const uint32_t a = sg.list[j];
        row |= ((my_m[a >> 12] >> ((a >> 7) & 30u)) & 1u) << (a & 31u);
    }
    return row;
}

// No hop scorer (the default): NR_BORDER_LEARNED needs the scorer's instantiation.
struct NrNoHopScore {
    __device__ float operator()(bool, const float (&)[NR_FEAT]) const { return 0.f; }
};

// FEAT: the learned scorer's instantiation (child features; with hop_score, the learned branch
// order).  hop_score(has, f) is warp-collective and returns the scorer's output for the lane's row.
template <int G, int W4, bool FEAT = false, class HopScore = NrNoHopScore>
__device__ __forceinline__ void nr_expand(const NrSmallGraph &g, const NrSmemGraph &sg,
                                          const uint32_t *my_m, bool valid, double mass, double eps,
                                          bool &has_child, uint32_t (&w)[4 * W4], double &cm,
                                          NrLaneAcc &acc, float (*feat)[NR_FEAT] = nullptr,
                                          NrRowIO *rio = nullptr, int border = NR_BORDER_SRC,
                                          const HopScore *hop_score = nullptr)
{
    constexpr int NW = 4 * W4;
    const int lane = threadIdx.x & 31;
    const int v = lane & (G - 1);
    const int gbase = lane & ~(G - 1);
    const bool leader = (v == 0);
    const int n = g.n, src = g.src, dst = g.dst;

    has_child = false;
    cm = 0.0;
    if (valid && leader) acc.nodes++;
    bool active = valid;
    if (active && eps > 0.0 && mass < eps) {          // main.cu:537-543
        if (leader) { acc.trunc++; nr_fix_add_mass(acc.et, mass); }
        active = false;
    }

    // not-down in-neighbour row of node v (carried in, or built from the mask)
    uint32_t row = 0;
    if (rio && rio->have) row = (active && v < n) ? rio->row_in : 0u;
    else if (active && v < n) row = nr_build_row(sg, my_m, v);

    // level-synchronous BFS, one ballot per level for all groups of the warp
    int par = -1, level = 0;
    const bool found = nr_group_bfs<G>(row, active, n, src, dst, par, level);
    if (active && !found && leader) acc.dead++;
    const bool live = active && found;
    const int L = live ? level : 0;                     // hops on the path

    // walk dst -> src: lane h of the group receives hop h = (u, v)
    int Lmax = L;
    for (int off = 16; off > 0; off >>= 1) Lmax = max(Lmax, __shfl_xor_sync(NR_FULL, Lmax, off));
    int hop_u = 0, hop_v = 0, cur = dst;
    for (int s = Lmax - 1; s >= 0; --s) {
        const int u = __shfl_sync(NR_FULL, par, gbase + (cur & (G - 1)));
        if (s < L) {
            if (v == s) { hop_u = u; hop_v = cur; }
            cur = u;
        }
    }
    int e_h = 0;
    bool unk = false;
    if (v < L) {
        e_h = sg.eid[hop_u * G + hop_v];
        unk = ((my_m[e_h >> 4] >> ((e_h & 15) << 1)) & 3u) == 3u;
    }

    // FP64 mass along the path in branch order (sequential, as the oracle); each hop lane
    // loads its own p first, so the chain only waits on shuffles and multiplies
    const double p_h = unk ? sg.p[e_h] : 1.0;
    double P = mass;
    int rank = v;                                       // the hop's place in the branch order
    if (border == NR_BORDER_SRC) {
        for (int h = 0; h < Lmax; ++h) {
            const double pe = __shfl_sync(NR_FULL, p_h, gbase + h);
            const bool u = __shfl_sync(NR_FULL, unk, gbase + h);
            if (h < L && u) {
                if (v == h) { cm = __dmul_rn(P, __dsub_rn(1.0, p_h)); has_child = true; }
                P = __dmul_rn(P, pe);
            }
        }
    } else {
        // rank among the group's UNKNOWN hops: dst side first, or by a key (stable in path
        // order, the oracle's insertion sort of the src -> dst path): p, or the learned key
        bool desc = (border == NR_BORDER_P_DESC);
        const bool rev = (border == NR_BORDER_DST);
        double key = p_h;
        if constexpr (FEAT) {
            if (hop_score && border == NR_BORDER_LEARNED) {
                // the scorer's residual reliability r of the subproblem with hop v down (the other
                // edges as in the parent); key (1 - p) x (1 - r): a likely, critical failure first
                uint32_t wh[NW];
#pragma unroll
                for (int k = 0; k < NW; ++k) wh[k] = my_m[k];
#pragma unroll
                for (int k = 0; k < NW; ++k)
                    if (unk && k == (e_h >> 4)) wh[k] &= ~(3u << ((e_h & 15) << 1));
                const uint32_t rs = __shfl_sync(NR_FULL, row, gbase + src);
                const uint32_t rd = __shfl_sync(NR_FULL, row, gbase + dst);
                const int ds = __popc(rs) - ((hop_u == src || hop_v == src) ? 1 : 0);
                const int dd = __popc(rd) - ((hop_u == dst || hop_v == dst) ? 1 : 0);
                float hf[NR_FEAT];
                nr_child_features<W4>(hf, wh, unk ? mass * (1.0 - p_h) : 0.0, mass, L, v, p_h, ds, dd, n, g.e);
                float r = (*hop_score)(unk, hf);
                r = (r >= 0.f) ? fminf(r, 1.f) : 0.f;  // a NaN estimate must not break the ranking
                key = (double)((1.f - (float)p_h) * (1.f - r));
                desc = true;
            }
        }
        rank = 0;
        for (int j = 0; j < Lmax; ++j) {
            const double kj = __shfl_sync(NR_FULL, key, gbase + j);
            const bool uj = __shfl_sync(NR_FULL, unk, gbase + j);
            const bool before = rev ? (j > v) : desc ? (kj > key || (kj == key && j < v)) : (kj < key || (kj == key && j < v));
            if (uj && j < L && before) ++rank;
        }
        for (int k = 0; k < Lmax; ++k) {
            const unsigned b = __ballot_sync(NR_FULL, unk && rank == k);
            const unsigned gb = (G == 32) ? b : ((b >> gbase) & ((1u << G) - 1u));
            const int hl = gb ? __ffs(gb) - 1 : 0;
            const double pe = __shfl_sync(NR_FULL, p_h, gbase + hl);
            if (gb) {
                if (v == hl) { cm = __dmul_rn(P, __dsub_rn(1.0, p_h)); has_child = true; }
                P = __dmul_rn(P, pe);
            }
        }
    }
    if (live && leader) { acc.leaves++; nr_fix_add_mass(acc.R, P); }

    // child of hop v: parent with the UNKNOWN hops before it in branch order up and hop v down
#pragma unroll
    for (int k = 0; k < NW; ++k) w[k] = my_m[k];
    for (int j = 0; j < Lmax; ++j) {
        const int e = __shfl_sync(NR_FULL, e_h, gbase + j);
        const bool u = __shfl_sync(NR_FULL, unk, gbase + j);
        const int rj = __shfl_sync(NR_FULL, rank, gbase + j);
        if (has_child && u && rj <= rank) {
            const int wi = e >> 4;
            const uint32_t bits = (rj < rank ? 2u : 3u) << ((e & 15) << 1);
#pragma unroll
            for (int k = 0; k < NW; ++k)
                if (k == wi) w[k] &= ~bits;
        }
    }
    if (rio) { rio->row = row; rio->cu = hop_u; rio->cv = hop_v; }
    if constexpr (FEAT) {
        // not-down degrees of src and dst in the child (the parent's rows minus the down edge)
        const uint32_t rs = __shfl_sync(NR_FULL, row, gbase + src);
        const uint32_t rd = __shfl_sync(NR_FULL, row, gbase + dst);
        if (has_child) {
            const int ds = __popc(rs) - ((hop_u == src || hop_v == src) ? 1 : 0);
            const int dd = __popc(rd) - ((hop_u == dst || hop_v == dst) ? 1 : 0);
            nr_child_features<W4>(*feat, w, cm, mass, L, rank, sg.p[e_h], ds, dd, n, g.e);
        }
    }
}


// Fork branching (workingPad/main.cu:303-430 with :550-565, FORK_BEST_EDGE):
// a path of up edges means the subproblem is connected, so its whole mass goes
// to R; else the optimistic path's UNKNOWN edge with the largest p (ties: the
// one nearest dst, which the reference's dst-first scan with a strict
// comparison keeps) gives two children: that edge down (held by the lane of its
// hop) and up (held by lane L of the group, L = hops on the path < G).
template <int G, int W4>
__device__ __forceinline__ void nr_expand_fork(const NrSmallGraph &g, const NrSmemGraph &sg,
                                               const uint32_t *my_m, bool valid, double mass, double eps,
                                               bool &has_child, uint32_t (&w)[4 * W4], double &cm,
                                               NrLaneAcc &acc)
{
    constexpr int NW = 4 * W4;
    const int lane = threadIdx.x & 31;
    const int v = lane & (G - 1);
    const int gbase = lane & ~(G - 1);
    const bool leader = (v == 0);
    const int n = g.n, src = g.src, dst = g.dst;

    has_child = false;
    cm = 0.0;
    if (valid && leader) acc.nodes++;
    bool active = valid;
    if (active && eps > 0.0 && mass < eps) {          // main.cu:537-543
        if (leader) { acc.trunc++; nr_fix_add_mass(acc.et, mass); }
        active = false;
    }
    // not-down and up in-neighbour rows of node v
    uint32_t row = 0, row_up = 0;
    if (active && v < n) {
        for (int j = sg.start[v]; j < sg.start[v + 1]; ++j) {
            const uint32_t a = sg.list[j];
            const uint32_t st = (my_m[a >> 12] >> ((a >> 7) & 30u)) & 3u;
            row |= (st & 1u) << (a & 31u);
            row_up |= (uint32_t)(st == 1u) << (a & 31u);
        }
    }
    int par, level;
    const bool connected = nr_group_bfs<G>(row_up, active, n, src, dst, par, level);
    if (active && connected && leader) { acc.leaves++; nr_fix_add_mass(acc.R, mass); }
    const bool go = active && !connected;
    const bool found = nr_group_bfs<G>(row, go, n, src, dst, par, level);
    if (go && !found && leader) acc.dead++;
    const bool live = go && found;
    const int L = live ? level : 0;

    // walk dst -> src: lane h of the group receives hop h = (u, v); hop L-1 is at dst
    int Lmax = L;
    for (int off = 16; off > 0; off >>= 1) Lmax = max(Lmax, __shfl_xor_sync(NR_FULL, Lmax, off));
    int hop_u = 0, hop_v = 0, cur = dst;
    for (int s = Lmax - 1; s >= 0; --s) {
        const int u = __shfl_sync(NR_FULL, par, gbase + (cur & (G - 1)));
        if (s < L) {
            if (v == s) { hop_u = u; hop_v = cur; }
            cur = u;
        }
    }
    int e_h = 0;
    bool unk = false;
    if (v < L) {
        e_h = sg.eid[hop_u * G + hop_v];
        unk = ((my_m[e_h >> 4] >> ((e_h & 15) << 1)) & 3u) == 3u;
    }
    // the pivot: largest p among the UNKNOWN hops, the highest hop index (nearest dst) on ties
    const double mp = unk ? sg.p[e_h] : -1.0;
    double best = mp;
    for (int off = G / 2; off > 0; off >>= 1) best = fmax(best, __shfl_xor_sync(NR_FULL, best, off, G));
    const unsigned cand = __ballot_sync(NR_FULL, unk && mp == best);
    const unsigned gc = (G == 32) ? cand : ((cand >> gbase) & ((1u << G) - 1u));
    const int hstar = gc ? 31 - __clz(gc) : 0;
    const int estar = __shfl_sync(NR_FULL, e_h, gbase + hstar);
    if (live && !gc && leader) { acc.leaves++; nr_fix_add_mass(acc.R, mass); }   // not reached: see above
    if (live && gc && (v == hstar || v == L)) {
        const bool down = (v == hstar);
        const double pe = sg.p[estar];
        cm = down ? __dmul_rn(mass, __dsub_rn(1.0, pe)) : __dmul_rn(mass, pe);
        const int wi = estar >> 4;
        const uint32_t clear = (down ? 3u : 2u) << ((estar & 15) << 1);
#pragma unroll
        for (int k = 0; k < NW; ++k) w[k] = (k == wi) ? (my_m[k] & ~clear) : my_m[k];
        has_child = true;
    }
}
