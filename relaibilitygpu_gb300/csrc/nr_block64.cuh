// nr_block64.cuh -- breadth-first waves of one instance on one block, one lane per subproblem,
// for undirected simple graphs of 33..64 nodes (64-bit rows) and up to 256 edges: a batch's
// middle-sized graphs, which otherwise take the wide engine's warp per subproblem.
//
// The schedule is the lane kernels' and the block kernel's (nr_block_lane.cuh): waves in two
// buffers per block, one shared-memory atomicAdd per warp step for the children's slots, the
// stop tests between waves in the oracle's order, the parent rule, path, children and
// FP64 products -- so every count and exact sum is the oracle's and the wide engine's.  What
// differs is the record: 64 rows of 64 bits would be 512 B, so a record is the mask and the
// mass only, and a lane rebuilds its record's not-down rows from the mask (one pass over the
// edges, both endpoints of every edge not down) into its shared-memory column before the BFS.
//
// Shared memory: the instance's p, edge endpoints and 64 x 64 edge-id table, then per warp the
// lanes' rows ([2 n_max][32] words: row u is words 2u, 2u + 1) and BFS levels ([2 n_max][32]:
// level l's 64-bit frontier in words 2l, 2l + 1, replaced by the path hops, then moved to
// words 0 .. L-1 for the branch order and the children).
#pragma once

#include "nr_block_lane.cuh"

#define NR_MID_MAX_N 64
#define NR_MID_MAX_W4 4
#define NR_MID_MAX_E (64 * NR_MID_MAX_W4)      // 256 edges: 32 mask words
#define NR_MID_MAX_WARPS 8

// hop words of 64-node graphs: 11-bit edge id, 6-bit nodes, a 9-bit sort key above bit 23
template <> struct NrHop<64> { static constexpr int EB = 11, NB = 6, KS = 23; };

__host__ __device__ constexpr int nr_mid_tab_bytes()
{
    return NR_MID_MAX_E * 8 + NR_MID_MAX_E * 2 + NR_MID_MAX_N * NR_MID_MAX_N * 2;
}

// dynamic shared memory of a launch whose largest graph has n_max nodes, with `warps` warps
__host__ __device__ inline size_t nr_mid_shm_bytes(int n_max, int warps)
{
    return (size_t)nr_mid_tab_bytes() + (size_t)warps * 4 * n_max * 32 * 4;
}

// The lane's not-down rows from its mask: row u holds bit v for every edge u - v not down.
template <int NW>
__device__ __forceinline__ void nr_mid_rows(uint32_t *my_rows, const uint32_t (&wc)[NW], const uint16_t *ends,
                                            int n, int ge)
{
    for (int k = 0; k < 2 * n; ++k) my_rows[32 * k] = 0u;
#pragma unroll
    for (int kw = 0; kw < NW; ++kw) {
        const uint32_t w = wc[kw];
        for (int i = 0; i < 16; ++i) {
            const int e = 16 * kw + i;
            if (e >= ge) break;
            if (((w >> (2 * i)) & 3u) == NR_EDGE_DOWN) continue;
            const uint32_t uv = ends[e];
            const int u = uv & 0xff, v = uv >> 8;
            my_rows[32 * (2 * u + (v >> 5))] |= 1u << (v & 31);
            my_rows[32 * (2 * v + (u >> 5))] |= 1u << (u & 31);
        }
    }
}

__device__ __forceinline__ unsigned long long nr_mid_row(const uint32_t *my_rows, int u)
{
    return (unsigned long long)my_rows[32 * (2 * u)] | ((unsigned long long)my_rows[32 * (2 * u + 1)] << 32);
}

// nr_lane_path with 64-bit rows: BFS from src (level l's frontier to words 2l, 2l + 1 of the
// level column; dst tested against the frontier first), then the walk dst -> src (the parent of
// a node on level l+1 is the smallest node of frontier l adjacent to it), the hops moved to
// words 0 .. L-1.  Same results and checks (bad: 2 levels, 3 parent, 4 edge id).
template <int NW>
__device__ __forceinline__ int nr_mid_path(const uint32_t *my_rows, uint32_t *my_lv, const uint32_t (&wc)[NW],
                                           const uint16_t *eid, int n, int ge, int src, int dst, bool active,
                                           bool &live, int &nch, int &bad)
{
    int L = 0;
    live = false;
    nch = 0;
    bad = 0;
    if (!active) return 0;
    if (src == dst) { live = true; return 0; }
    const unsigned long long rd = nr_mid_row(my_rows, dst);
    unsigned long long F = 1ull << src, vis = F;
    for (;;) {                                      // every level adds a node: at most n - 1 levels
        if (L >= n) { bad = 2; return 0; }
        my_lv[32 * (2 * L)] = (uint32_t)F;
        my_lv[32 * (2 * L + 1)] = (uint32_t)(F >> 32);
        if (rd & F) { ++L; live = true; break; }    // dst is on the next level
        unsigned long long nf = 0ull;
        for (unsigned long long t = F; t; t &= t - 1ull) nf |= nr_mid_row(my_rows, __ffsll((long long)t) - 1);
        nf &= ~vis;
        if (!nf) return 0;                          // a dead end has no path: no hops, no children
        vis |= nf;
        F = nf;
        ++L;
    }
    int x = dst;
    for (int l = L - 1; l >= 0; --l) {
        const unsigned long long fl = (unsigned long long)my_lv[32 * (2 * l)] |
                                      ((unsigned long long)my_lv[32 * (2 * l + 1)] << 32);
        const int u = __ffsll((long long)(nr_mid_row(my_rows, x) & fl)) - 1;
        if (u < 0 || u >= n) { bad = 3; return 0; }
        const uint32_t e = eid[u * NR_MID_MAX_N + x];
        if ((int)e >= ge) { bad = 4; return 0; }
        my_lv[32 * (2 * l)] = nr_hop_make<64>(e, (uint32_t)u, (uint32_t)x);
        nch += ((nr_pick(wc, (int)e >> 4) >> ((e & 15) << 1)) & 3u) == 3u;
        x = u;
    }
    for (int l = 1; l < L; ++l) my_lv[32 * l] = my_lv[32 * (2 * l)];   // (word 2l is read before l' > l writes)
    return L;
}

// The root record (warp 0): the mask from p (p <= 0 down, p >= 1 up, else unknown), mass 1.
template <int W4>
__device__ __forceinline__ void nr_mid_root(int ge, const double *tp, uint4 *mask, double *mass)
{
    const int lane = threadIdx.x & 31;
    uint32_t *rw = reinterpret_cast<uint32_t *>(mask);
#pragma unroll
    for (int e0 = 0; e0 < 64 * W4; e0 += 32) {
        const int e = e0 + lane;
        uint32_t v = 0u;
        if (e < ge) {
            const long long b = __double_as_longlong(tp[e]);
            const bool dn = b <= 0ll, up = b >= 0x3ff0000000000000ll;
            v = (uint32_t)(dn ? NR_EDGE_DOWN : up ? NR_EDGE_UP : NR_EDGE_UNKNOWN) << ((e & 15) << 1);
        }
        const uint32_t lo = __reduce_or_sync(NR_FULL, lane < 16 ? v : 0u);
        const uint32_t hi = __reduce_or_sync(NR_FULL, lane < 16 ? 0u : v);
        if (lane == 0) { rw[e0 >> 4] = lo; rw[(e0 >> 4) + 1] = hi; }
    }
    if (lane == 0) mass[0] = 1.0;
}

// P.pages * NR_PAGE records per wave buffer; P.row_words = 2 x the launch's largest node count.
template <int W4>
__global__ void __launch_bounds__(32 * NR_MID_MAX_WARPS, 1) nr_block64_kernel(NrWarpParams P)
{
    constexpr int NW = 4 * W4;
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_ii, s_bad;
    __shared__ unsigned long long s_next;          // children placed in the next wave (spilled ones too)
    __shared__ unsigned long long s_u64[NR_MID_MAX_WARPS];
    __shared__ NrFix s_fix[NR_MID_MAX_WARPS];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    double *tp = reinterpret_cast<double *>(smem);
    uint16_t *ends = reinterpret_cast<uint16_t *>(tp + NR_MID_MAX_E);
    uint16_t *eid = ends + NR_MID_MAX_E;
    const int RWD = P.row_words;
    uint32_t *my_rows = reinterpret_cast<uint32_t *>(smem + nr_mid_tab_bytes()) + (size_t)warp * 2 * RWD * 32 + lane;
    uint32_t *my_lv = my_rows + RWD * 32;

    const unsigned long long cap = (unsigned long long)P.pages * NR_PAGE;
    uint4 *mask_b = P.slab_mask + (size_t)blockIdx.x * 2 * cap * W4;
    double *mass_b = P.slab_mass + (size_t)blockIdx.x * 2 * cap;
    const bool use_eps = P.eps > 0.0;
    const bool use_units = P.target >= 1e-30;
    const float unit_scale = use_units ? __double2float_rd(1048576.0 / P.target) : 0.0f;
    const unsigned root_units = use_units ? min(__float2uint_rd(unit_scale), NR_LANE2_UNIT_CAP) : 0u;

    for (int round = 0;; ++round) {
        __syncthreads();                            // the last instance's reads of s_ii and the tables are done
        if (threadIdx.x == 0) {
            s_ii = round == 0 ? (int)blockIdx.x : atomicAdd(P.next_inst, 1) + (int)gridDim.x;
            s_bad = 0;
        }
        __syncthreads();
        const int ii = s_ii;
        if (ii >= P.n_inst) break;
        const NrSmallGraph g = P.inst[ii];
        {
            const unsigned char *gb = P.blob + g.blob_off;
            const double *gp = reinterpret_cast<const double *>(gb + g.off_p);
            const uint16_t *ge_ = reinterpret_cast<const uint16_t *>(gb + g.off_list);
            const uint32_t *gi = reinterpret_cast<const uint32_t *>(gb + g.off_eid);
            for (int e = threadIdx.x; e < g.e; e += blockDim.x) { tp[e] = gp[e]; ends[e] = ge_[e]; }
            for (int k = threadIdx.x; k < NR_MID_MAX_N * NR_MID_MAX_N / 2; k += blockDim.x)
                reinterpret_cast<uint32_t *>(eid)[k] = gi[k];
        }
        __syncthreads();
        const long long t0 = nr_globaltimer();
        if (warp == 0) nr_mid_root<W4>(g.e, tp, mask_b, mass_b);
        const int n = g.n, src = g.src, dst = g.dst, ge = g.e;
        NrLaneAcc acc;
        nr_acc_zero(acc);
        unsigned qunits = threadIdx.x == 0 ? root_units : 0u;   // lower bound of the queued mass
        unsigned long long n_in = 1, max_wave = 0;
        int waves = 0, check = 0;

        for (int wave = 0;; ++wave) {
            const int cur = wave & 1;
            const double *in_mass = mass_b + (size_t)cur * cap;
            // ---- stop tests between waves, in the oracle's order: empty queue, target width, budget ----
            const unsigned long long units = nr_u64_block_sum(use_units ? qunits : 0u, s_u64);
            const unsigned long long nodes = nr_u64_block_sum(acc.nodes, s_u64);
            int st = !check && n_in == 0 ? 0 : -1;         // an empty queue first, as in the oracle
            NrFix qs = nr_fix_zero();
            bool summed = false;
            if (!check && st < 0 && P.target > 0.0 && units <= NR_LANE2_UNITS) {
                for (unsigned long long r = threadIdx.x; r < n_in; r += blockDim.x)
                    nr_fix_add_mass(qs, __ldcg(in_mass + r));
                summed = true;
                NrFix w = qs;
                nr_fix_add(w, acc.et);
                nr_fix_add(w, acc.es);
                if (nr_fix_le(nr_fix_block_sum(w, s_fix), P.target_fix)) st = 1;
            }
            if (!check && st < 0 && P.max_nodes && nodes >= P.max_nodes) st = 3;
            if (!check && st < 0 && (waves > ge + 1 || (P.step_cap > 0 && waves >= P.step_cap))) check = 1;
            if (check || st >= 0) {
                if (!summed)
                    for (unsigned long long r = threadIdx.x; r < n_in; r += blockDim.x)
                        nr_fix_add_mass(qs, __ldcg(in_mass + r));
                const NrFix R = nr_fix_block_sum(acc.R, s_fix);
                const NrFix et = nr_fix_block_sum(acc.et, s_fix);
                const NrFix es_ = nr_fix_block_sum(acc.es, s_fix);
                const NrFix qm = nr_fix_block_sum(qs, s_fix);
                const unsigned long long leaves = nr_u64_block_sum(acc.leaves, s_u64);
                const unsigned long long dead = nr_u64_block_sum(acc.dead, s_u64);
                const unsigned long long trunc = nr_u64_block_sum(acc.trunc, s_u64);
                const unsigned long long spilled = nr_u64_block_sum(acc.spilled, s_u64);
                if (threadIdx.x == 0) {
                    NrWarpOut o;
                    o.R = check ? nr_fix_zero() : R; o.et = check ? nr_fix_zero() : et;
                    o.es = check ? nr_fix_zero() : es_; o.q = check ? nr_fix_zero() : qm;
                    o.nodes = nodes; o.leaves = leaves; o.dead = dead; o.trunc = trunc; o.spilled = spilled;
                    o.queued = check ? 0ull : n_in;
                    o.t_ns = nr_globaltimer() - t0;
                    o.waves = waves;
                    o.max_wave = check ? (unsigned long long)check : max_wave;
                    o.status = check ? NR_LANE_STATUS_CHECK : st;
                    P.out[P.inst_id[ii]] = o;
                }
                break;
            }

            // ---- one wave ----
            ++waves;
            if (n_in > max_wave) max_wave = n_in;
            qunits = 0u;
            if (threadIdx.x == 0) s_next = 0ull;
            __syncthreads();
            const uint4 *in_mask = mask_b + (size_t)cur * cap * W4;
            uint4 *out_mask = mask_b + (size_t)(cur ^ 1) * cap * W4;
            double *out_mass = mass_b + (size_t)(cur ^ 1) * cap;
            for (unsigned long long base = (unsigned long long)warp * 32; base < n_in;
                 base += (unsigned long long)nwarp * 32) {
                const unsigned long long idx = base + lane;
                const bool valid = idx < n_in;
                uint32_t wc[NW];
                double mass = 0.0;
                if (valid) {
#pragma unroll
                    for (int k = 0; k < W4; ++k) {
                        const uint4 q = __ldcg(in_mask + idx * W4 + k);
                        wc[4 * k] = q.x; wc[4 * k + 1] = q.y; wc[4 * k + 2] = q.z; wc[4 * k + 3] = q.w;
                    }
                    mass = __ldcg(in_mass + idx);
                } else {
#pragma unroll
                    for (int k = 0; k < NW; ++k) wc[k] = 0u;
                }
                bool active = valid;
                if (valid) {
                    acc.nodes++;
                    if (use_eps && mass < P.eps) {          // main.cu:537-543
                        acc.trunc++;
                        nr_fix_add_mass(acc.et, mass);
                        active = false;
                    }
                }
                if (active) nr_mid_rows<NW>(my_rows, wc, ends, n, ge);
                bool live;
                int nch, bad;
                const int L = nr_mid_path<NW>(my_rows, my_lv, wc, eid, n, ge, src, dst, active, live, nch, bad);
                if (bad) {                                  // an internal check failed: no children
                    atomicCAS(&s_bad, 0, bad);
                    nch = 0;
                    live = false;
                }
                if (P.border != NR_BORDER_SRC && L > 1 && !bad) nr_lane_branch_order<64>(my_lv, L, P.border, tp);
                if (active && !live && !bad) acc.dead++;

                int pre = nch;
#pragma unroll
                for (int off = 1; off < 32; off <<= 1) {
                    const int t = __shfl_up_sync(NR_FULL, pre, off);
                    if (lane >= off) pre += t;
                }
                const int total = __shfl_sync(NR_FULL, pre, 31);
                unsigned long long obase = 0;
                if (lane == 0 && total > 0) obase = atomicAdd(&s_next, (unsigned long long)total);
                obase = __shfl_sync(NR_FULL, obase, 0);
                unsigned long long q = obase + (unsigned long long)(pre - nch);
                double Pm = mass;
                unsigned qadd = 0u;
                for (int h = 0; h < L && !bad; ++h) {
                    const uint32_t hp = my_lv[32 * h];
                    const int e = nr_hop_e<64>(hp);
                    const int ew = e >> 4;
                    const uint32_t wv = nr_pick(wc, ew);
                    if (((wv >> ((e & 15) << 1)) & 3u) != 3u) continue;     // only UNKNOWN hops branch
                    const double pe = tp[e];
                    const double cm = __dmul_rn(Pm, __dsub_rn(1.0, pe));
                    Pm = __dmul_rn(Pm, pe);
                    if (q < cap) {
                        uint4 *d = out_mask + q * W4;
#pragma unroll
                        for (int kk = 0; kk < W4; ++kk)
                            d[kk] = make_uint4(wc[4 * kk], wc[4 * kk + 1], wc[4 * kk + 2], wc[4 * kk + 3]);
                        reinterpret_cast<uint32_t *>(d)[ew] = wv & ~(3u << ((e & 15) << 1));
                        out_mass[q] = cm;
                        qadd += min(__float2uint_rd(__fmul_rd(__double2float_rd(cm), unit_scale)), NR_LANE2_UNIT_CAP);
                    } else {                                // the wave buffer is full: mass to ESP
                        acc.spilled++;
                        nr_fix_add_mass(acc.es, cm);
                    }
                    ++q;
#pragma unroll
                    for (int kk = 0; kk < NW; ++kk)         // later children see hop h up
                        if (kk == ew) wc[kk] &= ~(2u << ((e & 15) << 1));
                }
                if (live) {
                    acc.leaves++;
                    nr_fix_add_mass(acc.R, Pm);
                }
                if (qadd) qunits = min(qunits + min(qadd, NR_LANE2_UNIT_CAP), NR_LANE2_UNIT_CAP);
                __syncwarp();                               // the rows and levels are rewritten by the next step
            }
            __syncthreads();                                // the wave's children are written
            n_in = min(s_next, cap);
            if (s_bad) check = s_bad;
        }
    }
}
