// nr_warp.cuh -- warp-per-instance engine for batches and small truncated runs.
//
// The reference runs one graph per process through a host-driven wave loop
// (workingPad/main.cu:963-1008).  Here each warp takes whole instances from
// a device counter and solves them with a private queue:
//   * subproblems live in the warp's own slab of HBM, in pages of 32 records
//     (16-byte mask blocks + FP64 mass);
//   * page chains are grouped into mass buckets (the bucketed max-mass
//     priority queue); chain heads, page counts, a free-page stack and a
//     bucket bitmap sit in the warp's shared memory, so queue bookkeeping
//     needs no atomics and no global synchronisation;
//   * wave mode (truncated runs): a wave takes the whole chain of the
//     fullest non-empty bucket; children land in fresh chains, so the set of
//     expanded subproblems, and the stop test between waves (ESP + queued
//     mass <= target), match the oracle's wave schedule exactly;
//   * page mode (exhaustive runs): one page at a time, depth-first, which
//     keeps the live queue small; results do not depend on the order.
// A warp that runs out of pages (or past max_nodes) either spills the child
// mass into ESP, as the reference does when its queue is full
// (main.cu:245-252), or marks the instance for the whole-GPU engine.
#pragma once

#include "nr_expand.cuh"
#include "nr_mlp.cuh"

#define NR_WARP_BLOCK 128        // default block: 4 warps
#define NR_WARP_BLOCK_MAX 256    // largest block the warp kernels are compiled for
#ifndef NR_WARP_MIN_BLOCKS
#define NR_WARP_MIN_BLOCKS 3     // resident 256-thread blocks per SM the register budget must allow
#endif
#define NR_PAGE 32
#define NR_WARP_STATUS_CHECK 4   // an internal check failed; max_wave holds which (host: NR_ERR_INTERNAL)

struct NrWarpOut {
    NrFix R, et, es, q;   // exact sums: leaves, eps-truncated, spilled, still queued
    unsigned long long nodes, leaves, dead, trunc, spilled, queued, max_wave;
    long long t_ns;       // device time from instance start to stop (target met or queue empty)
    int waves;
    int status;           // 0 queue empty, 1 target width met, 2 handed over, 3 budget reached
};

struct NrWarpParams {
    const unsigned char *blob;       // all instances' graph tables
    const NrSmallGraph *inst;        // [n_inst] (this class only)
    const int *inst_id;              // [n_inst] -> index into out
    int n_inst;
    int *next_inst;                  // work counter
    uint4 *slab_mask;                // [warps][pages*32][w4]
    double *slab_mass;               // [warps][pages*32]
    uint32_t *slab_rows;             // [warps][pages*32][G]: not-down in-neighbour rows (nullptr: none)
    int pages;                       // pages per warp
    int n_buckets;                   // multiple of 32, <= 256
    int shift;                       // bucket resolution (2^shift per octave); < 0 = one bucket
    int wave_mode;                   // 1: whole-bucket waves; 0: one page at a time
    int escalate;                    // 1: on overflow hand the instance to the grid engine
    double eps;
    double target;                   // stop once ESP + queued mass <= target (wave mode); 0 = off
    NrFix target_fix;                // the same target as an exact fixed-point number
    unsigned long long max_nodes;    // pop budget: page mode hands over, wave mode stops (0 = none)
    NrWarpOut *out;
    // learned variant only (nr_warp_kernel<G, W4, true>)
    int learned;                     // 1: bucket key = child mass x scorer output
    NrMlpDev mlp;
    float *dump_feat;                // optional: every child's features ...
    uint32_t *dump_mask;             // ... mask words (dump_stride words each) ...
    double *dump_mass;               // ... mass ...
    int *dump_inst;                  // ... and instance index
    unsigned long long *dump_count;
    unsigned long long dump_cap;
    int dump_stride;
    int inst_base;                   // index of this launch's instance 0 in the caller's batch
    int fork;                        // fork branching (informational: the FORK instantiation runs it)
    int border;                      // NR_BORDER_*: the order a path's UNKNOWN edges are branched in
    long long step_cap;              // lane kernels: steps before the self-check ends an instance
                                     // (0: NR_LANE_STEP_CAP; the failure-path tests set 1)
    int handover_pages;              // two-slot lane kernel: an instance whose next wave holds more
                                     // pages than this is handed over (status 2) to the block
                                     // kernel (nr_block_lane.cuh); 0 = never
    int row_words;                   // 64-bit-row block kernel (nr_block64.cuh): shared-memory words
                                     // a lane's rows take (and its BFS levels): 2 x the largest n
};

__device__ __forceinline__ unsigned long long nr_warp_sum_u64(unsigned long long x)
{
    for (int off = 16; off > 0; off >>= 1) x += __shfl_xor_sync(NR_FULL, x, off);
    return x;
}

// shared memory of one warp: staged items, bucket heads and bitmap, page metadata
struct NrWarpShm {
    uint32_t *masks;     // [K * 4 * W4]
    short *heads;        // [n_buckets]
    uint32_t *bitmap;    // [n_buckets / 32]
    short *pnext;        // [pages]
    unsigned char *pcnt; // [pages]
    short *freel;        // [pages]
};

// The learned branch order's hop scorer: the MLP on the warp's scratch (learned kernels only).
struct NrWarpHopScore {
    NrMlpDev M;
    uint32_t *scratch;
    float *y;
    __device__ float operator()(bool has, const float (&f)[NR_FEAT]) const
    {
        return nr_mlp_score_lanes(M, scratch, y, has, f);
    }
};

__host__ __device__ inline size_t nr_warp_shm_bytes(int K, int W4, int n_buckets, int pages, bool learn = false)
{
    size_t b = 32 * sizeof(NrLaneAcc);                             // per-lane sums and counters
    b += learn ? (size_t)(NR_MLP_WARP_WORDS + 16) * 4 : 0;         // scorer scratch + outputs
    b += (size_t)K * 4 * W4 * 4;
    b += (size_t)n_buckets * 2;
    b = (b + 3) & ~size_t(3);
    b += (size_t)(n_buckets / 32) * 4;
    b += (size_t)pages * 2;
    b += (size_t)pages;
    b = (b + 1) & ~size_t(1);
    b += (size_t)pages * 2;
    return (b + 15) & ~size_t(15);
}

// The per-lane sums and counters (updated a few times per subproblem) live in
// shared memory, which keeps the plain kernel for masks of up to 4 blocks at 80
// registers without spills: three 256-thread blocks, 24 warps, per SM.  Wider
// masks hold more words per lane (two blocks per SM), and the scorer's kernel
// needs its registers for the MLP.
// FORK instantiates fork branching (nr_expand_fork) in place of path branching.
template <int G, int W4, bool LEARN = false, bool FORK = false>
__global__ void __launch_bounds__(NR_WARP_BLOCK_MAX, LEARN ? 1 : (W4 <= 4 ? NR_WARP_MIN_BLOCKS : 2))
    nr_warp_kernel(NrWarpParams P)
{
    constexpr int K = 32 / G;
    constexpr int NW = 4 * W4;
    extern __shared__ __align__(16) unsigned char smem[];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int grp = lane / G, v = lane & (G - 1);
    const bool leader = (v == 0);
    const unsigned lt_mask = (1u << lane) - 1u;
    const int NB = P.n_buckets, NP = P.pages;

    NrWarpShm sh;
    uint32_t *mlp_scratch = nullptr;
    float *mlp_y = nullptr;
    NrLaneAcc *acc_base;
    {
        unsigned char *b = smem + (size_t)warp * nr_warp_shm_bytes(K, W4, NB, NP, LEARN);
        acc_base = reinterpret_cast<NrLaneAcc *>(b);
        b += 32 * sizeof(NrLaneAcc);
        size_t o = 0;
        if (LEARN) {
            mlp_scratch = reinterpret_cast<uint32_t *>(b);
            mlp_y = reinterpret_cast<float *>(b + (size_t)NR_MLP_WARP_WORDS * 4);
            o = (size_t)(NR_MLP_WARP_WORDS + 16) * 4;
        }
        sh.masks = reinterpret_cast<uint32_t *>(b + o); o += (size_t)K * NW * 4;
        sh.heads = reinterpret_cast<short *>(b + o); o += (size_t)NB * 2; o = (o + 3) & ~size_t(3);
        sh.bitmap = reinterpret_cast<uint32_t *>(b + o); o += (size_t)(NB / 32) * 4;
        sh.pnext = reinterpret_cast<short *>(b + o); o += (size_t)NP * 2;
        sh.pcnt = b + o; o += (size_t)NP; o = (o + 1) & ~size_t(1);
        sh.freel = reinterpret_cast<short *>(b + o);
    }
    uint32_t *my_m = sh.masks + grp * NW;
    const size_t gw = (size_t)blockIdx.x * (blockDim.x >> 5) + warp;
    uint4 *sl_mask = P.slab_mask + gw * (size_t)NP * NR_PAGE * W4;
    double *sl_mass = P.slab_mass + gw * (size_t)NP * NR_PAGE;
    uint32_t *sl_rows = P.slab_rows ? P.slab_rows + gw * (size_t)NP * NR_PAGE * G : nullptr;

    for (;;) {
        int ii = 0;
        if (lane == 0) ii = atomicAdd(P.next_inst, 1);
        ii = __shfl_sync(NR_FULL, ii, 0);
        if (ii >= P.n_inst) break;
        const NrSmallGraph g = P.inst[ii];
        const unsigned char *gb = P.blob + g.blob_off;         // this instance's p
        const unsigned char *gs = P.blob + g.struct_off;       // its topology's tables (maybe shared)
        NrSmemGraph sg;
        sg.p = reinterpret_cast<const double *>(gb + g.off_p);
        sg.eid = reinterpret_cast<const uint16_t *>(gs + g.off_eid);
        sg.start = reinterpret_cast<const int *>(gs + g.off_start);
        sg.list = reinterpret_cast<const uint32_t *>(gs + g.off_list);
        // rows travel with the records on simple graphs (the fork branching rebuilds its own)
        const int rows_mode = (FORK || !sl_rows) ? 0 : g.rows;
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
        {
            // root record from p: p <= 0 down, p >= 1 up, else unknown (main.cu:717-748);
            // 16 edges a word, each half-warp ORs one word together
            uint32_t *rw = reinterpret_cast<uint32_t *>(sl_mask + (size_t)rpg * NR_PAGE * W4);
            for (int e0 = 0; e0 < 64 * W4; e0 += 32) {
                const int e = e0 + lane;
                uint32_t v = 0u;
                if (e < g.e) {
                    const double pe = sg.p[e];
                    v = (uint32_t)((pe <= 0.0) ? NR_EDGE_DOWN : (pe >= 1.0) ? NR_EDGE_UP : NR_EDGE_UNKNOWN)
                        << ((e & 15) << 1);
                }
                v |= __shfl_xor_sync(NR_FULL, v, 8);
                v |= __shfl_xor_sync(NR_FULL, v, 4);
                v |= __shfl_xor_sync(NR_FULL, v, 2);
                v |= __shfl_xor_sync(NR_FULL, v, 1);
                if ((lane & 15) == 0) rw[(e0 >> 4) + (lane >> 4)] = v;
            }
        }
        if (lane == 0) sl_mass[(size_t)rpg * NR_PAGE] = 1.0;
        if (rows_mode && grp == 0) {
            // the root's rows: an arc u -> v is not down when p > 0 (its edge is up or unknown)
            uint32_t r = 0;
            if (v < g.n)
                for (int j = sg.start[v]; j < sg.start[v + 1]; ++j) {
                    const uint32_t a = sg.list[j];
                    if (sg.p[a >> 8] > 0.0) r |= 1u << (a & 31u);
                }
            sl_rows[(size_t)rpg * NR_PAGE * G + v] = r;
        }
        __syncwarp();

        NrLaneAcc &acc = acc_base[lane];
        nr_acc_zero(acc);
        NrFix qacc = (lane == 0) ? nr_fix_of(1.0) : nr_fix_zero();   // queued mass: this lane's pushes - pops
        long long qcount = (lane == 0) ? 1 : 0;
        int waves = 0, status = 0;
        unsigned long long max_wave = 0;
        bool abandon = false;
        long long t_stop = 0;

        for (;;) {
            // fullest (lowest-index) non-empty bucket; an empty queue ends the run before the other
            // tests, as in the oracle's wave loop (pathdecomp.c: empty, target width, budget)
            const uint32_t wb = (lane < NB / 32) ? sh.bitmap[lane] : 0u;
            const unsigned nz = __ballot_sync(NR_FULL, wb != 0u);
            if (!nz) break;
            if (P.wave_mode && P.target > 0.0) {     // exact: ESP + queued mass <= target
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
            const int bk = wi * 32 + __ffs(__shfl_sync(NR_FULL, wb, wi)) - 1;
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
            int walked = 0;                          // pages of this chain so far: at most NP
            for (int pg = chain; pg >= 0 && !abandon;) {
                if (++walked > NP) break;            // longer than the pool: the chain is corrupt
                const int cnt = sh.pcnt[pg];
                const int nxt = sh.pnext[pg];
                wave_items += cnt;
                for (int i0 = 0; i0 < cnt; i0 += K) {
                    const int idx = i0 + grp;
                    const bool valid = idx < cnt;
                    const size_t slot = (size_t)pg * NR_PAGE + idx;
                    if (valid && v < W4) reinterpret_cast<uint4 *>(my_m)[v] = sl_mask[slot * W4 + v];
                    NrRowIO rio;
                    rio.have = rows_mode != 0;
                    rio.row_in = (rows_mode && valid) ? sl_rows[slot * G + v] : 0u;
                    const double mass = valid ? sl_mass[slot] : 0.0;
                    if (valid && leader) { nr_fix_sub(qacc, nr_fix_of(mass)); qcount--; }
                    __syncwarp();

                    bool has_child;
                    uint32_t w[NW];
                    double cm;
                    float feat[NR_FEAT];
                    if constexpr (FORK)
                        nr_expand_fork<G, W4>(g, sg, my_m, valid, mass, P.eps, has_child, w, cm, acc);
                    else
                    {
                        const NrWarpHopScore hs{P.mlp, mlp_scratch, mlp_y};
                        nr_expand<G, W4, LEARN, NrWarpHopScore>(g, sg, my_m, valid, mass, P.eps, has_child, w, cm,
                                                                acc, LEARN ? &feat : nullptr, &rio, P.border,
                                                                LEARN ? &hs : nullptr);
                    }
                    double key = cm;
                    if constexpr (LEARN) {
                        const unsigned cbm = __ballot_sync(NR_FULL, has_child);
                        if (P.dump_feat && has_child) {     // training data: the child as it is queued
                            const unsigned long long d = atomicAdd(P.dump_count, 1ull);
                            if (d < P.dump_cap) {
#pragma unroll
                                for (int k = 0; k < NR_FEAT; ++k) P.dump_feat[d * NR_FEAT + k] = feat[k];
#pragma unroll
                                for (int k = 0; k < NW; ++k) P.dump_mask[d * P.dump_stride + k] = w[k];
                                P.dump_mass[d] = cm;
                                P.dump_inst[d] = P.inst_base + P.inst_id[ii];
                            }
                        }
                        if (P.learned && cbm) {             // score this step's children, 16 per tile
                            const int nch = __popc(cbm), rank = __popc(cbm & lt_mask);
                            for (int t = 0; t * 16 < nch; ++t) {
                                if (has_child && rank / 16 == t) {
#pragma unroll
                                    for (int k = 0; k < NR_FEAT / 2; ++k)
                                        mlp_scratch[(rank % 16) * 8 + k] = nr_pack_bf16(feat[2 * k], feat[2 * k + 1]);
                                }
                                nr_mlp_warp_infer(P.mlp, mlp_scratch, mlp_y);
                                if (has_child && rank / 16 == t) key = cm * (double)mlp_y[rank % 16];
                                __syncwarp();
                            }
                        }
                    }
                    const int cb = has_child ? nr_bucket(key, P.shift, NB) : 0;

                    unsigned pend = __ballot_sync(NR_FULL, has_child);
                    while (pend) {
                        const int b = __shfl_sync(NR_FULL, cb, __ffs(pend) - 1);
                        const unsigned m = __ballot_sync(NR_FULL, has_child && cb == b);
                        const int n = __popc(m);
                        int hA = -1, cA = 0, nA = 0, hB = -1;
                        if (lane == 0) {
                            const int h = sh.heads[b];
                            const int c = (h >= 0) ? sh.pcnt[h] : NR_PAGE;
                            nA = min(n, NR_PAGE - c);
                            if (nA > 0) { hA = h; cA = c; sh.pcnt[h] = (unsigned char)(c + nA); }
                            const int rest = n - nA;
                            if (rest > 0 && top > 0) {
                                hB = sh.freel[--top];
                                sh.pnext[hB] = (short)h;
                                sh.pcnt[hB] = (unsigned char)rest;
                                sh.heads[b] = (short)hB;
                                sh.bitmap[b >> 5] |= 1u << (b & 31);
                            }
                        }
                        top = __shfl_sync(NR_FULL, top, 0);
                        hA = __shfl_sync(NR_FULL, hA, 0);
                        cA = __shfl_sync(NR_FULL, cA, 0);
                        nA = __shfl_sync(NR_FULL, nA, 0);
                        hB = __shfl_sync(NR_FULL, hB, 0);
                        __syncwarp();
                        int s = -1;                       // this lane's child's slot
                        if (has_child && cb == b) {
                            const int r = __popc(m & lt_mask);
                            s = (r < nA) ? hA * NR_PAGE + cA + r : (hB >= 0 ? hB * NR_PAGE + (r - nA) : -1);
                            if (s >= 0) {
                                uint4 *d = sl_mask + (size_t)s * W4;
#pragma unroll
                                for (int k = 0; k < W4; ++k)
                                    d[k] = make_uint4(w[4 * k], w[4 * k + 1], w[4 * k + 2], w[4 * k + 3]);
                                sl_mass[s] = cm;
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
                        if (rows_mode) {
                            // the children's rows: the parent's, less the arcs of the child's down
                            // edge; one child of every group per step, lane v writes node v's row
                            const int gb = lane & ~(G - 1);
                            unsigned todo = (G == 32) ? m : ((m >> gb) & ((1u << G) - 1u));
                            while (__any_sync(NR_FULL, todo != 0u)) {
                                const int c = todo ? __ffs(todo) - 1 : 0;
                                const int sc = __shfl_sync(NR_FULL, s, gb + c);
                                const int cu = __shfl_sync(NR_FULL, rio.cu, gb + c);
                                const int cv = __shfl_sync(NR_FULL, rio.cv, gb + c);
                                if (todo && sc >= 0) {
                                    uint32_t rr = rio.row;
                                    if (v == cv) rr &= ~(1u << cu);
                                    if (rows_mode == 1 && v == cu) rr &= ~(1u << cv);
                                    sl_rows[(size_t)sc * G + v] = rr;
                                }
                                todo &= todo - 1u;
                            }
                        }
                        pend = __ballot_sync(NR_FULL, has_child);
                    }
                    abandon = __any_sync(NR_FULL, abandon);
                    if (abandon) break;
                }
                if (lane == 0) sh.freel[top++] = (short)pg;
                top = __shfl_sync(NR_FULL, top, 0);
                __syncwarp();
                pg = nxt;
            }
            if (walked > NP) { status = NR_WARP_STATUS_CHECK; max_wave = 6; break; }
            if (abandon) { status = 2; break; }
            if (wave_items > max_wave) max_wave = wave_items;
        }
        t_stop = nr_globaltimer() - t0;

        const NrFix R = nr_fix_warp_sum(acc.R), et = nr_fix_warp_sum(acc.et), es = nr_fix_warp_sum(acc.es);
        const NrFix qm = nr_fix_warp_sum(qacc);
        const unsigned long long nodes = nr_warp_sum_u64(acc.nodes), leaves = nr_warp_sum_u64(acc.leaves);
        const unsigned long long dead = nr_warp_sum_u64(acc.dead), trunc = nr_warp_sum_u64(acc.trunc);
        const unsigned long long spilled = nr_warp_sum_u64(acc.spilled);
        const unsigned long long queued = nr_warp_sum_u64((unsigned long long)qcount);
        if (lane == 0) {
            NrWarpOut o;
            o.R = R; o.et = et; o.es = es; o.q = qm;
            o.nodes = nodes; o.leaves = leaves; o.dead = dead; o.trunc = trunc; o.spilled = spilled;
            o.queued = queued; o.max_wave = max_wave; o.t_ns = t_stop; o.waves = waves; o.status = status;
            P.out[P.inst_id[ii]] = o;
        }
        __syncwarp();
    }
}
