// nr_lane2.cuh -- the lane kernel with several instances per warp (NS = 2 or 4), for
// breadth-first waves (one bucket) on undirected simple graphs of up to 16 nodes (16-bit
// rows, RB = 16), or up to 32 nodes with 32-bit rows (RB = 32: 128 B of rows a record, two
// slots a warp).
//
// nr_lane_kernel gives a warp one instance, and the first waves of an instance hold
// 1, 1, 2, 4, ... records: most lanes idle while every step pays its full fixed work,
// and a batch of a few thousand instances ends with a tail of warps on their last
// instance.  Here a warp carries NS instance slots.  A step takes the next page of as
// many slots' current waves as fit in 32 lanes, starting from a slot that rotates step
// by step; each taken page gets a contiguous range of lanes.  Each slot keeps
// its own wave structure -- its current wave's page chain, the chain its children go
// to, its own stop test between its waves -- so each instance follows exactly the
// schedule of the one-slot kernel and of the oracle; only the interleaving of the two
// instances' steps is new.  The slots share the warp's page pool, each limited to 1/NS
// of it, so a new instance always finds a page for its root.
#pragma once

#include "nr_lane.cuh"

// warp-uniform state of one instance slot, in shared memory (written by lane 0)
struct NrLaneSlot {
    long long t0;
    int ii;                 // instance (index into the class); -1 empty, -2 no instance left
    int n, src, dst, ge;
    int head;               // the chain the current wave's children go to (the next wave)
    int cur;                // next page of the current wave; -1: the wave is done
    int waves, used;        // waves started; pages held (current wave + next wave)
    unsigned wave_items, max_wave;
    int pad[3];             // 64 bytes
};

// a slot's copy of its instance's tables: p (simple graphs on <= 16 nodes: <= 120 edges; on
// <= 32 nodes: <= 496) and the edge-id table (n <= 8: 8 x 8 ids, n <= 16: 16 x 16, else 32 x 32)
__host__ __device__ constexpr int nr_lane2_max_e(int rb) { return rb == 16 ? 128 : 512; }
__host__ __device__ constexpr int nr_lane2_tab_bytes(int rb) { return nr_lane2_max_e(rb) * 8 + rb * rb * 2; }

__host__ __device__ inline size_t nr_lane2_shm_bytes(int pages, int slots, int rb = 16)
{
    size_t b = (size_t)slots * 32 * sizeof(NrLaneAcc);       // per slot, per lane sums
    b += (size_t)((rb == 16 ? 8 : 32) + rb) * 32 * 4;        // rows, hops, [word][lane]
    b += (size_t)slots * 32 * 4;                             // per slot, per lane: queued-mass lower bound (units)
    b += (size_t)slots * nr_lane2_tab_bytes(rb);             // per slot: p and edge ids
    b += (size_t)slots * sizeof(NrLaneSlot);
    b += (size_t)pages * 2;                                  // pnext
    b += (size_t)pages;                                      // pcnt
    b = (b + 1) & ~size_t(1);
    b += (size_t)pages * 2;                                  // free stack
    return (b + 15) & ~size_t(15);
}

// The root record of an instance at slot 0 of page rpg (the record nr_lane_root builds), from
// the slot's copy of p (tp, shared memory) and the topology's rows (r16: word `lane` of the
// table, preloaded).  Edge states come from p's bit pattern (p <= 0 down, p >= 1 up), with
// integer compares; each 16-edge mask word is one OR reduction over half the lanes' bits.
template <int W4, int RB = 16>
__device__ __forceinline__ void nr_lane2_root(const NrSmallGraph &g, const unsigned char *gs, const double *tp,
                                              uint32_t r16, uint4 *sl_mask, uint4 *sl_rows, double *sl_mass, int rpg)
{
    constexpr int RW = nr_lane_rw<RB>();
    const int lane = threadIdx.x & 31;
    uint32_t *rw = reinterpret_cast<uint32_t *>(sl_mask + (size_t)rpg * NR_PAGE * W4);
    bool down = false;
#pragma unroll
    for (int e0 = 0; e0 < 64 * W4; e0 += 32) {
        const int e = e0 + lane;
        uint32_t v = 0u;
        if (e < g.e) {
            const long long b = __double_as_longlong(tp[e]);
            const bool dn = b <= 0ll, up = b >= 0x3ff0000000000000ll;
            down = down || dn;
            v = (uint32_t)(dn ? NR_EDGE_DOWN : up ? NR_EDGE_UP : NR_EDGE_UNKNOWN) << ((e & 15) << 1);
        }
        const uint32_t lo = __reduce_or_sync(NR_FULL, lane < 16 ? v : 0u);
        const uint32_t hi = __reduce_or_sync(NR_FULL, lane < 16 ? 0u : v);
        if (lane == 0) { rw[e0 >> 4] = lo; rw[(e0 >> 4) + 1] = hi; }
    }
    uint32_t *rr = reinterpret_cast<uint32_t *>(sl_rows + (size_t)rpg * NR_PAGE * (RW / 4));
    if (!__any_sync(NR_FULL, down)) {
        if (lane < RW) rr[lane] = r16;
    } else {                                   // some edge is certainly down: gather the rows
        const int *start = reinterpret_cast<const int *>(gs + g.off_start);
        const uint32_t *list = reinterpret_cast<const uint32_t *>(gs + g.off_list);
        uint32_t r = 0;
        if (lane < g.n)
            for (int j = start[lane]; j < start[lane + 1]; ++j) {
                const uint32_t a = list[j];
                if (__double_as_longlong(tp[a >> 8]) > 0ll) r |= 1u << (a & 31u);
            }
        if constexpr (RB == 16) {
            const uint32_t hi = __shfl_down_sync(NR_FULL, r, 1);
            if (lane < 2 * RW && !(lane & 1)) rr[lane >> 1] = r | (hi << 16);
        } else {
            rr[lane] = r;                     // row `lane`; 0 past the nodes
        }
    }
    if (lane == 0) sl_mass[(size_t)rpg * NR_PAGE] = 1.0;
}

// the queued mass's lower bound is kept in units of target / 2^20, per lane and slot
#define NR_LANE2_UNITS (1u << 20)
#define NR_LANE2_UNIT_CAP (1u << 26)      // a lane's total saturates here: 32 lanes sum below 2^31

template <int W4, int NS, int RB = 16>
__global__ void __launch_bounds__(NR_WARP_BLOCK_MAX, 2) nr_lane2_kernel(NrWarpParams P)
{
    constexpr int NW = 4 * W4;
    constexpr int RW = nr_lane_rw<RB>();
    constexpr int TAB = nr_lane2_tab_bytes(RB), MAXE = nr_lane2_max_e(RB);
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int NP = P.pages;
    const int budget = max(1, NP / NS);       // pages one slot may hold

    unsigned char *wbase = smem + (size_t)warp * nr_lane2_shm_bytes(NP, NS, RB);
    NrLaneAcc *accs = reinterpret_cast<NrLaneAcc *>(wbase);                      // [slot * 32 + lane]
    uint32_t *my_rows = reinterpret_cast<uint32_t *>(wbase + NS * 32 * sizeof(NrLaneAcc)) + lane;
    uint32_t *my_hop = my_rows + RW * 32;
    unsigned *qlb = reinterpret_cast<unsigned *>(wbase + NS * 32 * sizeof(NrLaneAcc) +
                                                 (size_t)(RW + RB) * 32 * 4);  // [slot * 32 + lane]
    unsigned char *tabs = reinterpret_cast<unsigned char *>(qlb + NS * 32);                       // [slot]
    NrLaneSlot *slots = reinterpret_cast<NrLaneSlot *>(tabs + NS * TAB);
    short *pnext = reinterpret_cast<short *>(slots + NS);
    unsigned char *pcnt = reinterpret_cast<unsigned char *>(pnext + NP);
    short *freel = reinterpret_cast<short *>(pcnt + ((NP + 1) & ~1));

    const size_t gw = (size_t)blockIdx.x * (blockDim.x >> 5) + warp;
    uint4 *sl_mask = P.slab_mask + gw * (size_t)NP * NR_PAGE * W4;
    double *sl_mass = P.slab_mass + gw * (size_t)NP * NR_PAGE;
    uint4 *sl_rows = reinterpret_cast<uint4 *>(P.slab_rows) + gw * (size_t)NP * NR_PAGE * (RW / 4);
    const bool use_eps = P.eps > 0.0;
    const long long step_cap = P.step_cap > 0 ? P.step_cap : NR_LANE_STEP_CAP;
    // units: a child of mass m adds floor(m * 2^20 / target) (FP32, rounded down, <= the exact
    // value); a sum above 2^20 units is a queued mass above the target.  Targets below 1e-30
    // (a scale beyond FP32) take the exact test at every wave's end.
    const bool use_units = P.target >= 1e-30;
    const float unit_scale = use_units ? __double2float_rd(1048576.0 / P.target) : 0.0f;
    const unsigned root_units = use_units ? min(__float2uint_rd(unit_scale), NR_LANE2_UNIT_CAP) : 0u;
    const int nwarps = (int)(gridDim.x * (blockDim.x >> 5));
    unsigned fresh = (1u << NS) - 1u;          // slots whose first instance is still to take

    for (int p = lane; p < NP; p += 32) { freel[p] = (short)(NP - 1 - p); pnext[p] = -1; pcnt[p] = 0; }
    if (lane < NS) { slots[lane].ii = -1; slots[lane].cur = -1; slots[lane].head = -1; }
    int top = NP;
    long long steps = 0;
    __syncwarp();

    // end slot s's instance: its sums and counts to P.out, its pages back to the stack
    auto finish = [&](int s, int status, int check, const NrFix &qs, long long qn) {
        NrLaneAcc &A = accs[s * 32 + lane];
        const NrFix R = nr_fix_warp_sum(A.R), et = nr_fix_warp_sum_sparse(A.et), es_ = nr_fix_warp_sum_sparse(A.es);
        const NrFix qm = nr_fix_warp_sum_sparse(qs);
        const unsigned long long nodes = nr_warp_sum_u64r(A.nodes), leaves = nr_warp_sum_u64r(A.leaves);
        const unsigned long long dead = nr_warp_sum_u64r(A.dead), trunc = nr_warp_sum_u64r(A.trunc);
        const unsigned long long spilled = nr_warp_sum_u64r(A.spilled);
        const unsigned long long queued = nr_warp_sum_u64r((unsigned long long)qn);
        NrLaneSlot &S = slots[s];
        if (lane == 0) {
            NrWarpOut o;
            o.R = R; o.et = et; o.es = es_; o.q = qm;
            o.nodes = nodes; o.leaves = leaves; o.dead = dead; o.trunc = trunc; o.spilled = spilled;
            o.queued = queued; o.t_ns = nr_globaltimer() - S.t0; o.waves = S.waves;
            o.max_wave = check ? (unsigned long long)check : S.max_wave;
            o.status = check ? NR_LANE_STATUS_CHECK : status;
            P.out[P.inst_id[S.ii]] = o;
            for (int c = 0; c < 2; ++c)                       // both of its chains
                for (int pg = c ? S.head : S.cur; pg >= 0 && top < NP;) {
                    const int nx = pnext[pg];
                    pnext[pg] = -1;
                    freel[top++] = (short)pg;
                    pg = nx;
                }
            S.ii = -1; S.cur = -1; S.head = -1; S.used = 0;
        }
        top = __shfl_sync(NR_FULL, top, 0);
        __syncwarp();
    };

    for (;;) {
        // ---- slot upkeep (1): empty slots take instances.  Warp gw starts with instances
        // gw*NS .. gw*NS+NS-1 (no counter traffic as a batch starts); later ones come from the
        // counter, past those.  New instances are set up together: one round of table loads.
        {
            int ii_t[NS];
            bool any_new = false;
#pragma unroll
            for (int t = 0; t < NS; ++t) {
                ii_t[t] = -1;
                if (slots[t].ii != -1) continue;
                int ii;
                if (fresh & (1u << t)) {
                    ii = (int)gw * NS + t;
                    fresh &= ~(1u << t);
                } else if (nwarps * NS >= P.n_inst) {
                    ii = P.n_inst;                          // the first round took every instance
                } else {
                    int v = 0;
                    if (lane == 0) v = atomicAdd(P.next_inst, 1);
                    ii = __shfl_sync(NR_FULL, v, 0) + nwarps * NS;
                }
                if (ii >= P.n_inst) {
                    if (lane == 0) slots[t].ii = -2;
                    continue;
                }
                ii_t[t] = ii;
                any_new = true;
            }
            if (any_new) {
                NrSmallGraph g_t[NS];
                uint32_t r16[NS];
#pragma unroll
                for (int t = 0; t < NS; ++t)
                    if (ii_t[t] >= 0) g_t[t] = P.inst[ii_t[t]];
#pragma unroll
                for (int t = 0; t < NS; ++t) {          // the slots' tables, for the steps' lookups
                    r16[t] = 0u;
                    if (ii_t[t] < 0) continue;
                    const NrSmallGraph &g = g_t[t];
                    const unsigned char *gs = P.blob + g.struct_off;
                    double *tp = reinterpret_cast<double *>(tabs + t * TAB);
                    uint32_t *te = reinterpret_cast<uint32_t *>(tp + MAXE);
                    const double *gp = reinterpret_cast<const double *>(P.blob + g.blob_off + g.off_p);
                    const uint32_t *gi = reinterpret_cast<const uint32_t *>(gs + g.off_eid);
                    const int ew = (g.n <= 8 ? 8 : g.n <= 16 ? 16 : 32) * g.n / 2;   // edge-id words
                    for (int e = lane; e < g.e; e += 32) tp[e] = gp[e];
                    for (int k = lane; k < ew; k += 32) te[k] = gi[k];
                    if (lane < RW) r16[t] = reinterpret_cast<const uint32_t *>(gs + g.off_root_rows)[lane];
                }
                __syncwarp();
#pragma unroll
                for (int t = 0; t < NS; ++t) {
                    if (ii_t[t] < 0) continue;
                    const NrSmallGraph &g = g_t[t];
                    NrLaneSlot &S = slots[t];
                    const int rpg = freel[top - 1];        // a slot holds <= NP/NS pages: one is free
                    --top;
                    if (lane == 0) {
                        S.t0 = nr_globaltimer();
                        S.ii = ii_t[t];
                        S.n = g.n; S.src = g.src; S.dst = g.dst; S.ge = g.e;
                        S.waves = 0; S.wave_items = 0; S.max_wave = 0;
                        pcnt[rpg] = 1;
                        pnext[rpg] = -1;
                        S.head = rpg; S.cur = -1; S.used = 1;
                    }
                    nr_lane2_root<W4, RB>(g, P.blob + g.struct_off,
                                          reinterpret_cast<const double *>(tabs + t * TAB), r16[t],
                                      sl_mask, sl_rows, sl_mass, rpg);
                    nr_acc_zero(accs[t * 32 + lane]);
                    qlb[t * 32 + lane] = lane == 0 ? root_units : 0u;   // the root's mass is queued
                }
                __syncwarp();
            }
        }
        // ---- slot upkeep (2): slots whose wave is done (or whose first has not begun) ----
        for (int s = 0; s < NS; ++s) {
            NrLaneSlot &S = slots[s];
            if (S.ii < 0 || S.cur >= 0) continue;
            // slot s's wave is done (or its first not begun): the stop tests, in the oracle's and
            // the one-slot kernel's order (empty queue, target width, node budget).  The queued mass is the
            // next wave's chain.  Its exact sum is taken only where a test can end the run: a
            // lower bound of it (FP32 sums rounded down, kept as the children are written) above
            // the target already rules the width test out, as the exact test would.
            if (lane == 0 && S.wave_items > S.max_wave) S.max_wave = S.wave_items;
            NrLaneAcc &A = accs[s * 32 + lane];
            NrFix qs = nr_fix_zero();
            long long qn = 0;
            bool summed = false;
            auto chain_sum = [&]() -> bool {       // false: longer than the pool, the chain is corrupt
                int pg = S.head;
                for (int k = 0; pg >= 0 && k < NP; pg = pnext[pg], ++k)
                    if (lane < (int)pcnt[pg]) {
                        nr_fix_add_mass(qs, sl_mass[(size_t)pg * NR_PAGE + lane]);
                        qn++;
                    }
                summed = true;
                return pg < 0;
            };
            // an empty queue first, as in the oracle's wave loop
            int st = S.head < 0 ? 0 : -1;
            if (st < 0 && P.target > 0.0) {
                const unsigned units = use_units ? __reduce_add_sync(NR_FULL, qlb[s * 32 + lane]) : 0u;
                if (units <= NR_LANE2_UNITS) {
                    if (!chain_sum()) {
                        finish(s, 0, 6, nr_fix_zero(), 0);
                        continue;
                    }
                    NrFix w = qs;
                    nr_fix_add(w, A.et);
                    nr_fix_add(w, A.es);
                    w = nr_fix_warp_sum(w);
                    if (nr_fix_le(w, P.target_fix)) st = 1;
                }
            }
            if (st < 0 && P.max_nodes && nr_warp_sum_u64r(A.nodes) >= P.max_nodes) st = 3;
            __syncwarp();
            if (st < 0 && P.handover_pages > 0 && S.used > P.handover_pages) {
                // the next wave outgrows the warp: the block kernel runs the instance again
                // (queued reports the next wave's pages x 32, the host's largest-first order)
                finish(s, 2, 0, nr_fix_zero(), lane == 0 ? (long long)S.used * NR_PAGE : 0ll);
                continue;
            }
            if (st >= 0) {
                if (!summed && !chain_sum()) {
                    finish(s, 0, 6, nr_fix_zero(), 0);
                    continue;
                }
                finish(s, st, 0, qs, qn);
            } else {
                qlb[s * 32 + lane] = 0u;            // the next wave's children start a new chain
                if (lane == 0) { S.cur = S.head; S.head = -1; S.waves++; S.wave_items = 0; }
                __syncwarp();
            }
        }
        // ---- one step: the next page of as many slots' waves as fit in 32 lanes, starting
        // from a slot that rotates step by step (so no slot waits for long) ----
        int tpg[NS], toff[NS], tcnt[NS];          // per slot: page taken (-1 none), first lane, records
        int used_lanes = 0, empty_page = 0;
        bool all_done = true;
#pragma unroll
        for (int t = 0; t < NS; ++t) { tpg[t] = -1; toff[t] = 0; tcnt[t] = 0; all_done = all_done && slots[t].ii == -2; }
        if (all_done) break;
        const int t0 = (int)(steps % NS);
#pragma unroll
        for (int pass = 0; pass < 2; ++pass)        // slots t0 .. NS-1, then 0 .. t0-1
#pragma unroll
            for (int t = 0; t < NS; ++t) {          // (t is known at compile time: no local arrays)
                if ((t >= t0) != (pass == 0)) continue;
                const int cp = slots[t].ii >= 0 ? slots[t].cur : -1;
                if (cp < 0) continue;
                const int c = pcnt[cp];
                empty_page |= (c == 0);             // a chain page holds >= 1 record: checked, not assumed
                if (used_lanes + c > NR_PAGE) continue;
                tpg[t] = cp; toff[t] = used_lanes; tcnt[t] = c;
                used_lanes += c;
            }
        // Every pass counts toward the step bound, an idle one too, so the loop ends whatever
        // state the slots are in: past the bound (or on an empty chain page) the live slots end
        // with a check status, and the instances still to come end the same way at their first
        // pass.  (After the upkeep every live slot has a page of its current wave, so an idle
        // pass only follows instances ending: the next upkeep takes new ones or leaves.)
        if (++steps > step_cap || empty_page) {
            const int check = empty_page ? 5 : 1;
#pragma unroll 1
            for (int t = 0; t < NS; ++t)
                if (slots[t].ii >= 0) finish(t, 0, check, nr_fix_zero(), 0);
            continue;
        }
        if (used_lanes == 0) continue;              // the upkeep starts waves and instances
        int s = -1, pg = -1, idx = 0;
#pragma unroll
        for (int t = 0; t < NS; ++t)
            if (tpg[t] >= 0 && lane >= toff[t] && lane < toff[t] + tcnt[t]) { s = t; pg = tpg[t]; idx = lane - toff[t]; }
        const bool valid = s >= 0;
        const int sl = valid ? s : 0;
        const size_t slot = (size_t)(valid ? pg : 0) * NR_PAGE + idx;
        // 16-bit rows stay in registers too (the child writes copy them); 32-bit rows go
        // straight to the lane's shared-memory column
        constexpr int RWR = RB == 16 ? RW : 1;
        uint32_t wc[NW], rw[RWR];
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
                if constexpr (RB == 16) {
                    rw[4 * k] = q.x; rw[4 * k + 1] = q.y; rw[4 * k + 2] = q.z; rw[4 * k + 3] = q.w;
                } else {
                    my_rows[32 * (4 * k)] = q.x; my_rows[32 * (4 * k + 1)] = q.y;
                    my_rows[32 * (4 * k + 2)] = q.z; my_rows[32 * (4 * k + 3)] = q.w;
                }
            }
            mass = sl_mass[slot];
        } else {
#pragma unroll
            for (int k = 0; k < NW; ++k) wc[k] = 0u;
#pragma unroll
            for (int k = 0; k < RWR; ++k) rw[k] = 0u;
            if constexpr (RB == 32) {
#pragma unroll
                for (int k = 0; k < RW; ++k) my_rows[32 * k] = 0u;
            }
        }
        if constexpr (RB == 16) {
#pragma unroll
            for (int k = 0; k < RW; ++k) my_rows[32 * k] = rw[k];
        }
        __syncwarp();                               // every lane holds its record: the pages are free
        {
            // lane t < NS returns slot t's page to the stack (taken slots in slot order), one body
            // for all of them; every lane knows the new top
            int p0 = -1, at = top, cnt = 0;
#pragma unroll
            for (int t = 0; t < NS; ++t) {
                if (t == lane) { p0 = tpg[t]; cnt = tcnt[t]; }
                if (t < lane && tpg[t] >= 0) ++at;
            }
            if (lane < NS && p0 >= 0) {
                NrLaneSlot &T = slots[lane];
                T.cur = pnext[p0]; T.wave_items += cnt; T.used--;
                pnext[p0] = -1;
                freel[at] = (short)p0;
            }
#pragma unroll
            for (int t = 0; t < NS; ++t) top += tpg[t] >= 0;
        }
        __syncwarp();

        // the lane's instance
        const NrLaneSlot &S = slots[sl];
        const double *pt = reinterpret_cast<const double *>(tabs + sl * TAB);
        const uint16_t *eid = reinterpret_cast<const uint16_t *>(pt + MAXE);
        const int n = S.n, src = S.src, dst = S.dst, ge = S.ge;
        NrLaneAcc &acc = accs[sl * 32 + lane];

        bool active = valid;
        if (valid) {
            acc.nodes++;
            if (use_eps && mass < P.eps) {          // main.cu:537-543
                acc.trunc++;
                nr_fix_add_mass(acc.et, mass);
                active = false;
            }
        }
        bool live;
        int nch, bad;
        const int L = nr_lane_path<NW, RB>(my_rows, my_hop, wc, eid, n, ge, src, dst, active, live, nch, bad);
        if (P.border != NR_BORDER_SRC && L > 1) nr_lane_branch_order<RB>(my_hop, L, P.border, pt);
        if (active && !live && !bad) acc.dead++;
        {
            const unsigned bm = __ballot_sync(NR_FULL, bad != 0);
            if (bm) {                                   // an internal check failed: end both slots
                const int check = __shfl_sync(NR_FULL, bad, __ffs(bm) - 1);
                for (int t = 0; t < NS; ++t)
                    if (slots[t].ii >= 0) finish(t, 0, check, nr_fix_zero(), 0);
                continue;
            }
        }

        // children: a prefix over the lanes (slot 0's lanes first) places each slot's children
        // on that slot's next-wave chain, one allocation a slot
        int pre = nch;
#pragma unroll
        for (int off = 1; off < 32; off <<= 1) {
            const int t = __shfl_up_sync(NR_FULL, pre, off);
            if (lane >= off) pre += t;
        }
        // inclusive prefix before and at the end of each taken slot's lanes
        int tbeg[NS], tend[NS];
#pragma unroll
        for (int t = 0; t < NS; ++t) {
            const int e1 = __shfl_sync(NR_FULL, pre, tcnt[t] ? toff[t] + tcnt[t] - 1 : 0);
            const int b1 = __shfl_sync(NR_FULL, pre, toff[t] > 0 ? toff[t] - 1 : 0);
            tend[t] = tcnt[t] ? e1 : 0;
            tbeg[t] = (tcnt[t] && toff[t] > 0) ? b1 : 0;
        }
        pre -= nch;
        // Allocation, slot by slot: the head page's free records, then new pages from the free
        // stack.  Every lane computes it (its inputs are warp-uniform) and keeps its own slot's
        // part; lane t < NS then writes slot t's part, one body for all of them.
        int hA = -1, cA2 = 0, nA = 0, npg = 0, top0 = 0;
        int a_hd[NS], a_c[NS], a_n[NS], a_pg[NS], a_top[NS], a_want[NS];
#pragma unroll
        for (int t = 0; t < NS; ++t) {
            const int want = tend[t] - tbeg[t];
            const int hd = slots[t].head;
            const int c = (want > 0 && hd >= 0) ? (int)pcnt[hd] : NR_PAGE;
            const int na = want > 0 ? min(want, NR_PAGE - c) : 0;
            const int rest = want - na;
            const int np = want > 0 ? min(min((rest + NR_PAGE - 1) / NR_PAGE, top), max(0, budget - slots[t].used)) : 0;
            a_hd[t] = hd; a_c[t] = c; a_n[t] = na; a_pg[t] = np; a_top[t] = top; a_want[t] = want;
            top -= np;
            if (t == sl) { hA = na > 0 ? hd : -1; cA2 = c; nA = na; npg = np; top0 = a_top[t]; }
        }
        __syncwarp();                               // every lane has read the slots' state
        if (lane < NS) {
            int hd = -1, c = 0, na = 0, np = 0, t0p = 0, want = 0;
#pragma unroll
            for (int t = 0; t < NS; ++t)
                if (t == lane) { hd = a_hd[t]; c = a_c[t]; na = a_n[t]; np = a_pg[t]; t0p = a_top[t]; want = a_want[t]; }
            if (na > 0) pcnt[hd] = (unsigned char)(c + na);
            const int rest = want - na;
            int prev = hd;
            for (int i = 0; i < np; ++i) {
                const int pgi = freel[t0p - 1 - i];
                pnext[pgi] = (short)prev;
                pcnt[pgi] = (unsigned char)min(NR_PAGE, rest - NR_PAGE * i);
                prev = pgi;
            }
            if (np > 0) { slots[lane].head = prev; slots[lane].used += np; }
        }
        int q = pre;                                // this lane's first child, within its slot
#pragma unroll
        for (int t = 0; t < NS; ++t)
            if (t == sl) q -= tbeg[t];
        double Pm = mass;
        unsigned qadd = 0u;                         // lower bound of the mass this lane queues, in units
        for (int h = 0; h < L; ++h) {
            const uint32_t hp = my_hop[32 * h];
            const int e = nr_hop_e<RB>(hp);
            const int ew = e >> 4;
            const uint32_t wv = nr_pick(wc, ew);
            if (((wv >> ((e & 15) << 1)) & 3u) != 3u) continue;
            const int cu = nr_hop_u<RB>(hp), cv = nr_hop_x<RB>(hp);
            const double pe = pt[e];
            const double cm = __dmul_rn(Pm, __dsub_rn(1.0, pe));
            Pm = __dmul_rn(Pm, pe);
            int sc = -1;
            if (q < nA) {
                sc = hA * NR_PAGE + cA2 + q;
            } else {
                const int r = q - nA;
                if ((r >> 5) < npg) sc = freel[top0 - 1 - (r >> 5)] * NR_PAGE + (r & 31);
            }
            ++q;
            if (sc >= 0) {
                if constexpr (RB == 16)
                    nr_lane_write_child<W4>(sl_mask, sl_rows, sl_mass, sc, wc, rw, my_rows, e, wv, cu, cv, cm);
                else
                    nr_lane_write_child32<W4>(sl_mask, sl_rows, sl_mass, sc, wc, my_rows, e, wv, cu, cv, cm);
                qadd += min(__float2uint_rd(__fmul_rd(__double2float_rd(cm), unit_scale)), NR_LANE2_UNIT_CAP);
            } else {                                  // the slot's pages are full: mass to ESP
                acc.spilled++;
                nr_fix_add_mass(acc.es, cm);
            }
#pragma unroll
            for (int kk = 0; kk < NW; ++kk)            // later children see hop h up
                if (kk == ew) wc[kk] &= ~(2u << ((e & 15) << 1));
        }
        if (live) {
            acc.leaves++;
            nr_fix_add_mass(acc.R, Pm);
        }
        if (qadd) qlb[sl * 32 + lane] = min(qlb[sl * 32 + lane] + min(qadd, NR_LANE2_UNIT_CAP), NR_LANE2_UNIT_CAP);
        __syncwarp();
    }
}
