// nr_grid_lane.cuh -- whole-GPU wave engine with one lane per subproblem, for one
// undirected simple graph of up to 16 nodes (16-bit rows, RB = 16) or up to 32 nodes (32-bit
// rows, RB = 32: 128 B of rows a record), path branching.
//
// nr_grid_kernel spreads a subproblem over a lane group (a lane per node: the
// not-down rows rebuilt from the mask, one ballot per BFS level), two K10
// subproblems a warp step.  Here the lane kernels' step runs inside the same
// wave loop: a record carries its subproblem's 16 not-down rows (16 bits each,
// 32 B) beside the mask and the mass, each lane expands one record of the
// wave (bit-set BFS over the rows, nr_lane_path), and a child's rows are its
// parent's less the down edge -- so a warp step takes 32 records.  The parent
// rule, the path, the children and the FP64 products are the lane kernels',
// which are those of the lane-group kernel and the oracle; only the order of
// the children in the next wave's buffer differs, and exhaustive and
// eps-truncated totals and exact sums do not depend on it.
//
// Waves: ping-pong buffers (mask blocks, masses, rows), one warp-aggregated
// atomicAdd per warp step for the children's slots, the bounded grid barrier
// between waves; a slot at or past the capacity spills its child's mass into
// ESP (main.cu:245-252), as in nr_grid_kernel.
#pragma once

#include "nr_lane.cuh"

// shared memory: the staged graph tables, then per warp the lanes' rows [RW][32] and hops [RB][32]
__host__ __device__ inline size_t nr_grid_lane_shm_bytes(int blob_bytes, int warps, int rb = 16)
{
    return (((size_t)blob_bytes + 15) & ~size_t(15)) +
           (size_t)warps * ((rb == 16 ? 8 : 32) + rb) * 32 * sizeof(uint32_t);
}

template <int W4, int RB = 16>
__global__ void __launch_bounds__(NR_BLOCK_THREADS) nr_grid_lane_kernel(NrGridParams P)
{
    constexpr int NW = 4 * W4;
    constexpr int RW = nr_lane_rw<RB>();
    extern __shared__ __align__(16) unsigned char smem[];
    const NrSmallGraph g = P.g;
    nr_stage_blob(smem, P.blob, g.blob_bytes);
    __syncthreads();
    const double *pt = reinterpret_cast<const double *>(smem + g.off_p);
    const uint16_t *eid = reinterpret_cast<const uint16_t *>(smem + g.off_eid);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *my_rows = reinterpret_cast<uint32_t *>(smem + ((g.blob_bytes + 15) & ~15)) +
                        (size_t)warp * (RW + RB) * 32 + lane;                // word k at my_rows[32 k]
    uint32_t *my_hop = my_rows + RW * 32;                                      // level l at my_hop[32 l]
    const unsigned long long gw = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + warp;
    const unsigned long long TW = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long cap = P.capacity;
    const bool use_eps = P.eps > 0.0;
    const int n = g.n, src = g.src, dst = g.dst, ge = g.e;

    NrLaneAcc acc;
    nr_acc_zero(acc);

    for (int wave = 0; wave < P.max_waves; ++wave) {
        if (P.test_fault == 1 && blockIdx.x == 0) break;   // tests: the others' barrier waits run out
        unsigned long long n_in = *(volatile unsigned long long *)&P.wave_count[wave];
        if (n_in > cap) n_in = cap;
        if (n_in == 0) break;
        const uint4 *in_mask = P.mask[wave & 1];
        const double *in_mass = P.mass[wave & 1];
        const uint4 *in_rows = P.rows[wave & 1];
        uint4 *out_mask = P.mask[(wave + 1) & 1];
        double *out_mass = P.mass[(wave + 1) & 1];
        uint4 *out_rows = P.rows[(wave + 1) & 1];
        unsigned long long *out_count = &P.wave_count[wave + 1];

        for (unsigned long long base = gw * 32; base < n_in; base += TW * 32) {
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
                if (use_eps && mass < P.eps) {              // main.cu:537-543
                    acc.trunc++;
                    nr_fix_add_mass(acc.et, mass);
                    active = false;
                }
            }
            bool live;
            int nch, bad;
            const int L = nr_lane_path<NW, RB>(my_rows, my_hop, wc, eid, n, ge, src, dst, active, live, nch, bad);
            if (bad) {                                      // an internal check failed: no children
                atomicOr(P.status, NR_DEV_ERR_BOUNDS);
                nch = 0;
                live = false;
            }
            if (P.border != NR_BORDER_SRC && L > 1 && !bad) nr_lane_branch_order<RB>(my_hop, L, P.border, pt);
            if (active && !live && !bad) acc.dead++;

            // the warp's children take one range of the next wave's slots
            int pre = nch;
#pragma unroll
            for (int off = 1; off < 32; off <<= 1) {
                const int t = __shfl_up_sync(NR_FULL, pre, off);
                if (lane >= off) pre += t;
            }
            const int total = __shfl_sync(NR_FULL, pre, 31);
            unsigned long long obase = 0;
            if (lane == 0 && total > 0) obase = atomicAdd(out_count, (unsigned long long)total);
            obase = __shfl_sync(NR_FULL, obase, 0);
            unsigned long long q = obase + (unsigned long long)(pre - nch);
            double Pm = mass;
            for (int h = 0; h < L && !bad; ++h) {
                const uint32_t hp = my_hop[32 * h];
                const int e = nr_hop_e<RB>(hp);
                const int ew = e >> 4;
                const uint32_t wv = nr_pick(wc, ew);
                if (((wv >> ((e & 15) << 1)) & 3u) != 3u) continue;     // only UNKNOWN hops branch
                const double pe = pt[e];
                const double cm = __dmul_rn(Pm, __dsub_rn(1.0, pe));
                Pm = __dmul_rn(Pm, pe);
                if (q < cap) {
                    if constexpr (RB == 16)
                        nr_lane_write_child<W4>(out_mask, out_rows, out_mass, (int)q, wc, rw, my_rows, e, wv,
                                                nr_hop_u<RB>(hp), nr_hop_x<RB>(hp), cm);
                    else
                        nr_lane_write_child32<W4>(out_mask, out_rows, out_mass, (int)q, wc, my_rows, e, wv,
                                                  nr_hop_u<RB>(hp), nr_hop_x<RB>(hp), cm);
                } else {                                    // queue full: mass to ESP (main.cu:245-252)
                    acc.spilled++;
                    nr_fix_add_mass(acc.es, cm);
                }
                ++q;
#pragma unroll
                for (int kk = 0; kk < NW; ++kk)             // later children see hop h up
                    if (kk == ew) wc[kk] &= ~(2u << ((e & 15) << 1));
            }
            if (live) {
                acc.leaves++;
                nr_fix_add_mass(acc.R, Pm);
            }
            __syncwarp();
        }
        if (!nr_grid_sync(P.bar_count, P.bar_gen, P.status, P.timeout_ns)) break;
        if (wave + 1 == P.max_waves && threadIdx.x == 0 && blockIdx.x == 0 &&
            *(volatile unsigned long long *)&P.wave_count[wave + 1] != 0)
            atomicOr(P.status, NR_DEV_ERR_WAVES);
    }
    nr_block_partial(P.partials + blockIdx.x, acc.R, acc.et, acc.es, nr_fix_zero(), acc.nodes, acc.leaves, acc.dead,
                     acc.trunc, acc.spilled);
}
