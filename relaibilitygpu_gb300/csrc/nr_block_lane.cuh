// nr_block_lane.cuh -- breadth-first waves of one instance on one block, one lane per
// subproblem, for undirected simple graphs of up to 16 nodes (16-bit rows, RB = 16) or up to
// 32 nodes (32-bit rows, RB = 32): the instances of a batch whose waves outgrow a warp.
//
// nr_lane2_kernel runs an instance on one warp, 32 records a step.  In a batch of uneven
// instances a few of them run waves of tens of thousands of records, and the launch ends
// with their warps stepping alone while the rest of the GPU idles.  The two-slot kernel
// therefore hands an instance over at a wave boundary once its next wave holds more than
// P.handover_pages pages (status 2), and this kernel runs it again from its root on a whole
// block: each warp takes 32 records of the current wave at a time, the children go to the
// block's next-wave buffer (one shared-memory atomicAdd per warp step places a warp's
// children), and the block meets at the end of every wave for the stop tests.  Waves, stop
// tests (in the oracle's order: empty queue, target width, node budget), parent rule, path,
// children and FP64 products are the lane kernels', so every count and exact sum is
// what the two-slot kernel (and the oracle) reports; only the order of the children inside a
// wave is new, and nothing depends on it but which children spill when a wave outgrows the
// buffer.
//
// Blocks are persistent: block b starts with instance b and takes the next ones from the
// launch's counter.  Each owns two wave buffers of P.pages * NR_PAGE records (mask blocks,
// rows, mass) in P.slab_*; a child past the buffer spills its mass into ESP.
#pragma once

#include "nr_lane2.cuh"

// 16 warps an instance, one block per SM (128 registers): the largest instances' chains of waves
// are the launch's tail, and 8-warp blocks two per SM took 3-7 % longer on the uneven batch
#define NR_BLOCK_LANE_THREADS 512
#define NR_BLOCK_LANE_WARPS (NR_BLOCK_LANE_THREADS / 32)

// dynamic shared memory: the instance's p and edge-id tables, then per warp the lanes' rows
// [RW][32] and hops [RB][32]
__host__ __device__ inline size_t nr_block_lane_shm_bytes(int rb)
{
    return (size_t)nr_lane2_tab_bytes(rb) + (size_t)NR_BLOCK_LANE_WARPS * ((rb == 16 ? 8 : 32) + rb) * 32 * 4;
}

// bytes of one wave record: mask blocks, mass, rows
__host__ __device__ inline size_t nr_block_lane_rec_bytes(int w4, int rb)
{
    return 16 * (size_t)w4 + 8 + (rb == 16 ? 32 : 128);
}

// exact block total of a per-thread fixed-point value, returned on every thread (the block's
// threads all call it; s holds one value per warp)
__device__ __forceinline__ NrFix nr_fix_block_sum(const NrFix &a, NrFix *s)
{
    const NrFix w = nr_fix_warp_sum(a);
    __syncthreads();                                // earlier readers of s are done
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = w;
    __syncthreads();
    NrFix t = nr_fix_zero();
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) nr_fix_add(t, s[i]);
    return t;
}

__device__ __forceinline__ unsigned long long nr_u64_block_sum(unsigned long long x, unsigned long long *s)
{
    const unsigned long long w = nr_warp_sum_u64r(x);
    __syncthreads();
    if ((threadIdx.x & 31) == 0) s[threadIdx.x >> 5] = w;
    __syncthreads();
    unsigned long long t = 0;
    for (int i = 0; i < (int)(blockDim.x >> 5); ++i) t += s[i];
    return t;
}

template <int W4, int RB>
__global__ void __launch_bounds__(NR_BLOCK_LANE_THREADS, 1) nr_block_lane_kernel(NrWarpParams P)
{
    constexpr int NW = 4 * W4;
    constexpr int RW = nr_lane_rw<RB>();
    constexpr int MAXE = nr_lane2_max_e(RB);
    extern __shared__ __align__(16) unsigned char smem[];
    __shared__ int s_ii, s_bad;
    __shared__ unsigned long long s_next;          // children placed in the next wave (spilled ones too)
    __shared__ unsigned long long s_u64[NR_BLOCK_LANE_WARPS];
    __shared__ NrFix s_fix[NR_BLOCK_LANE_WARPS];

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nwarp = blockDim.x >> 5;
    double *tp = reinterpret_cast<double *>(smem);
    const uint16_t *eid = reinterpret_cast<const uint16_t *>(tp + MAXE);
    uint32_t *my_rows = reinterpret_cast<uint32_t *>(smem + nr_lane2_tab_bytes(RB)) +
                        (size_t)warp * (RW + RB) * 32 + lane;                  // word k at my_rows[32 k]
    uint32_t *my_hop = my_rows + RW * 32;                                      // level l at my_hop[32 l]

    const unsigned long long cap = (unsigned long long)P.pages * NR_PAGE;      // records per wave buffer
    uint4 *mask_b = P.slab_mask + (size_t)blockIdx.x * 2 * cap * W4;           // buffer k at + k * cap * W4
    double *mass_b = P.slab_mass + (size_t)blockIdx.x * 2 * cap;
    uint4 *rows_b = reinterpret_cast<uint4 *>(P.slab_rows) + (size_t)blockIdx.x * 2 * cap * (RW / 4);
    const bool use_eps = P.eps > 0.0;
    // the queued mass's lower bound, in units of target / 2^20, as in the two-slot kernel
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
        const unsigned char *gs = P.blob + g.struct_off;
        {
            const double *gp = reinterpret_cast<const double *>(P.blob + g.blob_off + g.off_p);
            const uint32_t *gi = reinterpret_cast<const uint32_t *>(gs + g.off_eid);
            const int ew = (g.n <= 8 ? 8 : g.n <= 16 ? 16 : 32) * g.n / 2;   // edge-id words
            for (int e = threadIdx.x; e < g.e; e += blockDim.x) tp[e] = gp[e];
            for (int k = threadIdx.x; k < ew; k += blockDim.x) reinterpret_cast<uint32_t *>(tp + MAXE)[k] = gi[k];
        }
        __syncthreads();
        const long long t0 = nr_globaltimer();
        if (warp == 0) {
            const uint32_t r16 = lane < RW ? reinterpret_cast<const uint32_t *>(gs + g.off_root_rows)[lane] : 0u;
            nr_lane2_root<W4, RB>(g, gs, tp, r16, mask_b, rows_b, mass_b, 0);
        }
        const int n = g.n, src = g.src, dst = g.dst, ge = g.e;
        NrLaneAcc acc;
        nr_acc_zero(acc);
        unsigned qunits = threadIdx.x == 0 ? root_units : 0u;   // lower bound of the queued mass
        unsigned long long n_in = 1, max_wave = 0;
        int waves = 0, check = 0;
        // (the root's global stores are visible to the block after the stop tests' barriers)

        for (int wave = 0;; ++wave) {
            const int cur = wave & 1;
            const double *in_mass = mass_b + (size_t)cur * cap;
            // ---- stop tests between waves, in the oracle's order: empty queue, target width, budget ----
            const unsigned long long units = nr_u64_block_sum(use_units ? qunits : 0u, s_u64);
            const unsigned long long nodes = nr_u64_block_sum(acc.nodes, s_u64);
            int st = !check && n_in == 0 ? 0 : -1;         // an empty queue first, as in the oracle
            NrFix qs = nr_fix_zero();                   // this thread's share of the queued mass
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
            // self-checks: a failed internal check; more waves than a path decomposition can have
            // (every child has one more edge down than its parent)
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
            const uint4 *in_rows = rows_b + (size_t)cur * cap * (RW / 4);
            uint4 *out_mask = mask_b + (size_t)(cur ^ 1) * cap * W4;
            double *out_mass = mass_b + (size_t)(cur ^ 1) * cap;
            uint4 *out_rows = rows_b + (size_t)(cur ^ 1) * cap * (RW / 4);
            for (unsigned long long base = (unsigned long long)warp * 32; base < n_in;
                 base += (unsigned long long)nwarp * 32) {
                const unsigned long long idx = base + lane;
                const bool valid = idx < n_in;
                // 16-bit rows stay in registers too (the child writes copy them); 32-bit rows go
                // straight to the lane's shared-memory column
                constexpr int RWR = RB == 16 ? RW : 1;
                uint32_t wc[NW], rw[RWR];
                double mass = 0.0;
                if (valid) {
#pragma unroll
                    for (int k = 0; k < W4; ++k) {
                        const uint4 q = __ldcg(in_mask + idx * W4 + k);
                        wc[4 * k] = q.x; wc[4 * k + 1] = q.y; wc[4 * k + 2] = q.z; wc[4 * k + 3] = q.w;
                    }
#pragma unroll
                    for (int k = 0; k < RW / 4; ++k) {
                        const uint4 q = __ldcg(in_rows + idx * (RW / 4) + k);
                        if constexpr (RB == 16) {
                            rw[4 * k] = q.x; rw[4 * k + 1] = q.y; rw[4 * k + 2] = q.z; rw[4 * k + 3] = q.w;
                        } else {
                            my_rows[32 * (4 * k)] = q.x; my_rows[32 * (4 * k + 1)] = q.y;
                            my_rows[32 * (4 * k + 2)] = q.z; my_rows[32 * (4 * k + 3)] = q.w;
                        }
                    }
                    mass = __ldcg(in_mass + idx);
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
                __syncwarp();

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
                if (bad) {                                  // an internal check failed: no children
                    atomicCAS(&s_bad, 0, bad);
                    nch = 0;
                    live = false;
                }
                if (P.border != NR_BORDER_SRC && L > 1 && !bad) nr_lane_branch_order<RB>(my_hop, L, P.border, tp);
                if (active && !live && !bad) acc.dead++;

                // the warp's children take one range of the next wave's buffer
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
                unsigned qadd = 0u;                         // lower bound of the mass queued here, in units
                for (int h = 0; h < L && !bad; ++h) {
                    const uint32_t hp = my_hop[32 * h];
                    const int e = nr_hop_e<RB>(hp);
                    const int ew = e >> 4;
                    const uint32_t wv = nr_pick(wc, ew);
                    if (((wv >> ((e & 15) << 1)) & 3u) != 3u) continue;     // only UNKNOWN hops branch
                    const double pe = tp[e];
                    const double cm = __dmul_rn(Pm, __dsub_rn(1.0, pe));
                    Pm = __dmul_rn(Pm, pe);
                    if (q < cap) {
                        if constexpr (RB == 16)
                            nr_lane_write_child<W4>(out_mask, out_rows, out_mass, (int)q, wc, rw, my_rows, e, wv,
                                                    nr_hop_u<RB>(hp), nr_hop_x<RB>(hp), cm);
                        else
                            nr_lane_write_child32<W4>(out_mask, out_rows, out_mass, (int)q, wc, my_rows, e, wv,
                                                      nr_hop_u<RB>(hp), nr_hop_x<RB>(hp), cm);
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
                __syncwarp();                               // my_rows / my_hop are rewritten by the next step
            }
            __syncthreads();                                // the wave's children are written
            n_in = min(s_next, cap);
            if (s_bad) check = s_bad;
        }
    }
}
