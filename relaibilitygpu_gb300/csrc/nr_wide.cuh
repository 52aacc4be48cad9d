// nr_wide.cuh -- whole-GPU engine for graphs with 33..1024 nodes.
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
// record is written with coalesced stores.  Waves, the grid barrier, the
// wave counters and the block partials work as in nr_grid.cuh.
//
// With a target width the run stops before the first wave at which
// ESP + queued mass <= target (the oracle's wave schedule with one bucket):
// at the end of a wave every block writes its exact share of that width
// (its ESP so far plus the mass it pushed) to one of two alternating slots,
// and after the grid barrier every block adds all shares and takes the same
// decision.  The pushed mass of the last wave run is the queued mass at the stop.
#pragma once

#include "nr_expand.cuh"

#define NR_WIDE_MAX_N 1024
#define NR_WIDE_MAX_W4 16
#define NR_WIDE_BLOCK 128

// Graph tables of one wide instance: p[E], q[E] (double), row_ptr[n+1] (int),
// arcs[n_arcs] (u32 = eid << 10 | head).  Offsets from the blob start, 16-byte aligned.
struct NrWideGraph {
    int n, e, w4, src, dst, n_arcs, nwd;
    int off_p, off_q, off_row, off_arc, blob_bytes;
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
    int target_on;              // stop at ESP + queued <= target_fix
    NrFix target_fix;
    NrFix *wpart;               // [2][gridDim.x] per-block width shares, alternating slots
    int *stop_wave;             // waves run before the target stop, or -1
};

// per-warp shared memory: mask words, frontier / next / visited bitmasks,
// packed parents, frontier list, path hops.  Rounded to 16 bytes: each
// warp's region starts with the mask, which is written with 16-byte stores.
__host__ __device__ inline size_t nr_wide_warp_shm(int n, int w4)
{
    return ((((size_t)4 * w4 + 3 * 32 + 3 * (size_t)n) * 4) + 15) & ~(size_t)15;
}

template <int W4>
__global__ void __launch_bounds__(NR_WIDE_BLOCK) nr_grid_wide_kernel(NrGridWideParams P)
{
    constexpr int NW = 4 * W4;
    extern __shared__ __align__(16) unsigned char smem[];
    const NrWideGraph g = P.g;
    nr_stage_blob(smem, P.blob, g.blob_bytes);
    __syncthreads();
    const double *p = reinterpret_cast<const double *>(smem + g.off_p);
    const double *q = reinterpret_cast<const double *>(smem + g.off_q);
    const int *row = reinterpret_cast<const int *>(smem + g.off_row);
    const uint32_t *arc = reinterpret_cast<const uint32_t *>(smem + g.off_arc);

    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    uint32_t *ws = reinterpret_cast<uint32_t *>(smem + g.blob_bytes + (size_t)warp * nr_wide_warp_shm(g.n, W4));
    uint32_t *m = ws;                       // [NW] mask words of the current subproblem
    uint32_t *F = m + NW;                   // [32] frontier
    uint32_t *NF = F + 32;                  // [32] next frontier
    uint32_t *VIS = NF + 32;                // [32] visited
    uint32_t *par = VIS + 32;               // [n] (parent << 16) | edge
    uint32_t *list = par + g.n;             // [n] frontier nodes
    uint32_t *hops = list + g.n;            // [n] path edges, dst side first
    const int n = g.n, nwd = g.nwd, src = g.src, dst = g.dst;
    const unsigned long long gw = (unsigned long long)blockIdx.x * (blockDim.x >> 5) + warp;
    const unsigned long long TW = (unsigned long long)gridDim.x * (blockDim.x >> 5);
    const unsigned long long cap = P.capacity;

    NrFix R = nr_fix_zero(), et = nr_fix_zero(), es = nr_fix_zero();
    // lane 0: mass this warp queued in the last wave run (the root counts as queued by
    // block 0's first warp, for a stop before the first wave)
    NrFix pushed = (blockIdx.x == 0 && threadIdx.x == 0) ? nr_fix_of(1.0) : nr_fix_zero();
    unsigned long long nodes = 0, leaves = 0, dead = 0, trunc = 0, spilled = 0;

    for (int wave = 0; wave < P.max_waves; ++wave) {
        unsigned long long n_in = *(volatile unsigned long long *)&P.wave_count[wave];
        if (n_in > cap) n_in = cap;
        if (n_in == 0) break;
        if (P.target_on) {
            NrFix width = nr_fix_zero();
            if (wave == 0) {
                width = nr_fix_of(1.0);                         // the root alone is queued
            } else {
                const NrFix *slot = P.wpart + (size_t)((wave - 1) & 1) * gridDim.x;
                for (unsigned b = threadIdx.x; b < gridDim.x; b += blockDim.x) {
                    NrFix v;                                    // written by other blocks: read from L2
                    v.w0 = __ldcg(&slot[b].w0);
                    v.w1 = __ldcg(&slot[b].w1);
                    v.w2 = __ldcg(&slot[b].w2);
                    nr_fix_add(width, v);
                }
                width = nr_block_fix_sum(width);
            }
            if (nr_fix_le(width, P.target_fix)) {
                if (threadIdx.x == 0 && blockIdx.x == 0) *P.stop_wave = wave;
                break;
            }
            pushed = nr_fix_zero();
        }
        const uint4 *in_mask = P.mask[wave & 1];
        const double *in_mass = P.mass[wave & 1];
        uint4 *out_mask = P.mask[(wave + 1) & 1];
        double *out_mass = P.mass[(wave + 1) & 1];
        unsigned long long *out_count = &P.wave_count[wave + 1];

        for (unsigned long long idx = gw; idx < n_in; idx += TW) {
            if (lane < W4) reinterpret_cast<uint4 *>(m)[lane] = __ldcg(in_mask + idx * W4 + lane);
            const double mass = __ldcg(in_mass + idx);
            if (lane == 0) nodes++;
            __syncwarp();
            if (P.eps > 0.0 && mass < P.eps) {          // main.cu:537-543
                if (lane == 0) { trunc++; nr_fix_add_mass(et, mass); }
                __syncwarp();
                continue;
            }
            // ---- BFS from src over not-down arcs ----
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
            bool found = (src == dst);
            int L = 0;
            while (!found) {
                // compact the frontier into list[]
                const uint32_t fw = (lane < nwd) ? F[lane] : 0u;
                const int cnt = __popc(fw);
                int pre = cnt;
                for (int off = 1; off < 32; off <<= 1) {
                    const int t = __shfl_up_sync(NR_FULL, pre, off);
                    if (lane >= off) pre += t;
                }
                const int total = __shfl_sync(NR_FULL, pre, 31);
                if (total == 0) break;
                int o = pre - cnt;
                for (uint32_t b = fw; b; b &= b - 1) list[o++] = (uint32_t)(lane * 32 + __ffs(b) - 1);
                for (int i = lane; i < nwd; i += 32) NF[i] = 0u;
                __syncwarp();
                for (int i = lane; i < total; i += 32) {
                    const uint32_t u = list[i];
                    for (int j = row[u]; j < row[u + 1]; ++j) {
                        const uint32_t a = arc[j];
                        const uint32_t v = a & 1023u, e = a >> 10;
                        if (((m[e >> 4] >> ((e & 15) << 1)) & 1u) && !((VIS[v >> 5] >> (v & 31)) & 1u)) {
                            atomicOr(&NF[v >> 5], 1u << (v & 31));
                            atomicMin(&par[v], (u << 16) | e);
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
                ++L;
                found = (VIS[dst >> 5] >> (dst & 31)) & 1u;
                if (!__any_sync(NR_FULL, any)) break;
            }
            if (!found) {
                if (lane == 0) dead++;
                __syncwarp();
                continue;
            }
            // ---- path: hops[] from dst back to src (L hops) ----
            if (lane == 0) {
                int v = dst, h = 0;
                while (v != src && h < n) {
                    const uint32_t pe = par[v];
                    hops[h++] = pe & 0xffffu;
                    v = (int)(pe >> 16);
                }
                L = h;
            }
            L = __shfl_sync(NR_FULL, L, 0);
            __syncwarp();
            // number of UNKNOWN hops -> one slot range for all children
            int unk = 0;
            for (int h = lane; h < L; h += 32) {
                const uint32_t e = hops[h];
                unk += ((m[e >> 4] >> ((e & 15) << 1)) & 3u) == 3u;
            }
            for (int off = 16; off > 0; off >>= 1) unk += __shfl_xor_sync(NR_FULL, unk, off);
            unsigned long long base = 0;
            if (lane == 0 && unk > 0) base = atomicAdd(out_count, (unsigned long long)unk);
            base = __shfl_sync(NR_FULL, base, 0);
            // children in hop order, src side first; lanes own mask words
            uint32_t w0 = (lane < NW) ? m[lane] : 0u;
            uint32_t w1 = (lane + 32 < NW) ? m[lane + 32] : 0u;
            double Pm = mass;
            int k = 0;
            for (int h = L - 1; h >= 0; --h) {
                const uint32_t e = hops[h];
                const int sh = (int)(e & 15u) << 1;
                const int wi = (int)(e >> 4);
                if (((m[wi] >> sh) & 3u) != 3u) continue;          // only UNKNOWN hops branch
                const unsigned long long slot = base + (unsigned long long)k;
                const double cm = __dmul_rn(Pm, q[e]);
                if (slot < cap) {
                    uint32_t *dstw = reinterpret_cast<uint32_t *>(out_mask + slot * W4);
                    if (lane < NW) __stcg(dstw + lane, (lane == wi) ? (w0 & ~(3u << sh)) : w0);
                    if (lane + 32 < NW) __stcg(dstw + lane + 32, (lane + 32 == wi) ? (w1 & ~(3u << sh)) : w1);
                    if (lane == 0) {
                        __stcg(out_mass + slot, cm);
                        if (P.target_on) nr_fix_add_mass(pushed, cm);
                    }
                } else if (lane == 0) {                             // queue full (main.cu:245-252)
                    spilled++;
                    nr_fix_add_mass(es, cm);
                }
                if (lane == wi) w0 &= ~(2u << sh);                  // this hop is up in later children
                if (lane + 32 == wi) w1 &= ~(2u << sh);
                Pm = __dmul_rn(Pm, p[e]);
                ++k;
            }
            if (lane == 0) { leaves++; nr_fix_add_mass(R, Pm); }
            __syncwarp();
        }
        if (P.target_on) {
            // this block's share of the width after the wave: ESP so far + mass it queued
            NrFix share = nr_fix_zero();
            if (lane == 0) {
                share = et;
                nr_fix_add(share, es);
                nr_fix_add(share, pushed);
            }
            share = nr_block_fix_sum(share);
            if (threadIdx.x == 0) {
                NrFix *dst = P.wpart + (size_t)(wave & 1) * gridDim.x + blockIdx.x;
                __stcg(&dst->w0, share.w0);
                __stcg(&dst->w1, share.w1);
                __stcg(&dst->w2, share.w2);
            }
        }
        if (!nr_grid_sync(P.bar_count, P.bar_gen, P.status, P.timeout_ns)) break;
        if (wave + 1 == P.max_waves && threadIdx.x == 0 && blockIdx.x == 0 &&
            *(volatile unsigned long long *)&P.wave_count[wave + 1] != 0)
            atomicOr(P.status, NR_DEV_ERR_WAVES);
    }
    nr_block_partial(P.partials + blockIdx.x, R, et, es, P.target_on ? pushed : nr_fix_zero(), nodes, leaves,
                     dead, trunc, spilled);
}
