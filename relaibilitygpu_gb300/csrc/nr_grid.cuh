// nr_grid.cuh -- whole-GPU engine for one instance with n_nodes <= 32.
//
// One cooperative persistent launch replaces the reference's host wave loop
// (workingPad/main.cu:963-1008: one factoring_kernel launch, a device sync
// and three small memcpys per wave).  Waves run back to back inside the
// kernel, separated by a bounded grid barrier.  Wave k reads the ping-pong
// buffer k%2 and appends children to the other one through one
// warp-aggregated atomicAdd per warp step; the per-wave counters stay on the
// device, so the host only reads them once at the end.  Subproblems are
// 16-byte-block mask records (coalesced 128-bit loads and stores) with the
// FP64 masses in a separate array.
#pragma once

#include "nr_expand.cuh"

// FORK instantiates fork branching (nr_expand_fork) in place of path branching.
template <int G, int W4, bool FORK = false>
__global__ void __launch_bounds__(NR_BLOCK_THREADS) nr_grid_kernel(NrGridParams P)
{
    constexpr int K = 32 / G;
    constexpr int NW = 4 * W4;
    extern __shared__ __align__(16) unsigned char smem[];
    const NrSmallGraph g = P.g;
    unsigned char *s_blob = smem;
    uint32_t *s_masks = reinterpret_cast<uint32_t *>(smem + g.blob_bytes);

    nr_stage_blob(s_blob, P.blob, g.blob_bytes);
    __syncthreads();
    const NrSmemGraph sg = nr_smem_graph(s_blob, g);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int grp = lane / G, v = lane & (G - 1);
    const unsigned lt_mask = (1u << lane) - 1u;
    uint32_t *my_m = s_masks + (warp * K + grp) * NW;
    const unsigned long long gw = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + warp;
    const unsigned long long TW = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long cap = P.capacity;

    NrLaneAcc acc;
    nr_acc_zero(acc);

    for (int wave = 0; wave < P.max_waves; ++wave) {
        if (P.test_fault == 1 && blockIdx.x == 0) break;   // tests: the others' barrier waits run out
        unsigned long long n_in = *(volatile unsigned long long *)&P.wave_count[wave];
        if (n_in > cap) n_in = cap;
        if (n_in == 0) break;
        const uint4 *in_mask = P.mask[wave & 1];
        const double *in_mass = P.mass[wave & 1];
        uint4 *out_mask = P.mask[(wave + 1) & 1];
        double *out_mass = P.mass[(wave + 1) & 1];
        unsigned long long *out_count = &P.wave_count[wave + 1];

        for (unsigned long long base = gw * K; base < n_in; base += TW * K) {
            const unsigned long long idx = base + grp;
            const bool valid = idx < n_in;
            if (valid && v < W4) reinterpret_cast<uint4 *>(my_m)[v] = __ldcg(in_mask + idx * W4 + v);
            const double mass = valid ? __ldcg(in_mass + idx) : 0.0;
            __syncwarp();

            bool has_child;
            uint32_t w[NW];
            double cm;
            if constexpr (FORK)
                nr_expand_fork<G, W4>(g, sg, my_m, valid, mass, P.eps, has_child, w, cm, acc);
            else
                nr_expand<G, W4>(g, sg, my_m, valid, mass, P.eps, has_child, w, cm, acc, nullptr, nullptr, P.border);

            const unsigned cb = __ballot_sync(NR_FULL, has_child);
            if (cb) {
                unsigned long long obase = 0;
                if (lane == 0) obase = atomicAdd(out_count, (unsigned long long)__popc(cb));
                obase = __shfl_sync(NR_FULL, obase, 0);
                if (has_child) {
                    const unsigned long long slot = obase + __popc(cb & lt_mask);
                    if (slot < cap) {
                        uint4 *dstm = out_mask + slot * W4;
#pragma unroll
                        for (int k = 0; k < W4; ++k)
                            __stcg(dstm + k, make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]));
                        __stcg(out_mass + slot, cm);
                    } else {                       // queue full: mass to ESP (main.cu:245-252)
                        acc.spilled++;
                        nr_fix_add_mass(acc.es, cm);
                    }
                }
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
