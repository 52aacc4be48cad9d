// nr_batch.cu -- the warp engine's batch runtime behind the C ABI (include/nr.h): table
// building, launches and results of nr_reliability_batch, nr_batch_submit / nr_batch_wait,
// matrix batches, the autotuner, the learned scorer's entries.  No reference counterpart: the
// reference runs one graph per process (workingPad/main.cu:795-1072).

#include "nr_host.h"

// Sets *flag when any of the n doubles is a NaN (integer test of the bit pattern).
__global__ void nr_nan_scan_kernel(const unsigned long long *p, size_t n, int *flag)
{
    int hit = 0;
    for (size_t i = (size_t)blockIdx.x * blockDim.x + threadIdx.x; i < n; i += (size_t)gridDim.x * blockDim.x)
        hit |= (p[i] & 0x7fffffffffffffffull) > 0x7ff0000000000000ull;
    if (__syncthreads_or(hit) && threadIdx.x == 0) *flag = 1;
}

static cudaError_t nr_launch_nan_scan(const double *p, size_t n, int *flag, cudaStream_t s)
{
    if (!n) return cudaSuccess;
    const int block = 256;
    const int grid = (int)std::min<size_t>((n + block - 1) / block, 1024);
    nr_nan_scan_kernel<<<grid, block, 0, s>>>(reinterpret_cast<const unsigned long long *>(p), n, flag);
    return cudaGetLastError();
}


// ---------------------------------------------------------------------------
// warp-per-instance engine (nr_warp.cuh)
// ---------------------------------------------------------------------------


WarpRunCfg warp_cfg(const nr_options *o, uint64_t capacity, bool exhaustive)
{
    WarpRunCfg w;
    w.eps = o->truncation_eps > 0 ? o->truncation_eps : 0.0;
    w.target = o->target_width > 0 ? o->target_width : 0.0;
    if (exhaustive) {
        w.wave_mode = 0; w.shift = -1; w.n_buckets = 32; w.escalate = 1;
        w.max_nodes = o->max_nodes ? o->max_nodes : (1ull << 21);
    } else {
        // NR_ORDER_WAVES: breadth-first waves, i.e. one bucket, whatever bucket_shift says
        w.wave_mode = 1; w.shift = (o->order == NR_ORDER_WAVES) ? -1 : o->bucket_shift;
        w.escalate = 0; w.max_nodes = o->max_nodes;
        w.learned = (o->order == NR_ORDER_LEARNED);
        int nb = o->n_buckets > 0 ? o->n_buckets : 256;
        nb = std::min(1024, (nb + 31) / 32 * 32);
        w.n_buckets = nb;
    }
    w.fork = (o->branching == NR_BRANCH_FORK);
    w.step_cap = (o->test_fault == 2) ? 1 : 0;
    w.border = o->branch_order;
    w.handover_pages = o->handover_pages < 0 ? 0 : o->handover_pages > 0 ? o->handover_pages : NR_HANDOVER_PAGES;
    w.lane = (o->small_kernel != NR_SMALL_GROUP);
    w.lane2 = (o->small_kernel == NR_SMALL_AUTO) && w.wave_mode && w.shift < 0;
    w.lane_slots = (o->lane_slots == 4) ? 4 : 2;
    w.warps_per_block = (o->warps_per_block >= 1 && o->warps_per_block <= NR_WARP_BLOCK_MAX / 32)
                            ? o->warps_per_block : NR_WARP_BLOCK / 32;
    if (capacity == 0) w.pages = o->pages_per_warp > 0 ? std::min(8192, std::max(4, o->pages_per_warp)) : 512;
    else w.pages = (int)std::min<uint64_t>(8192, std::max<uint64_t>(4, (capacity + NR_PAGE - 1) / NR_PAGE));
    return w;
}

static void fill_from_warp(const NrWarpOut &w, const WarpRunCfg &cfg, int W4, nr_result *r)
{
    NrFix esp = w.et;
    nr_fix_add(esp, w.es);
    nr_fix_add(esp, w.q);          // exact pushes - pops: zero on an empty queue
    r->R = nr_fix_to_double_host(w.R);
    r->esp = nr_fix_to_double_host(esp);
    r->R_plus_esp = r->R + r->esp;
    r->trunc_bound = r->R > 0 ? r->esp / r->R : r->esp;
    r->nodes = w.nodes; r->leaves = w.leaves; r->dead_ends = w.dead; r->truncated = w.trunc;
    r->spilled = w.spilled; r->paths = w.leaves + w.spilled; r->queued = w.queued;
    r->iterations = w.waves;
    r->max_queue_items = w.max_wave;
    r->item_bytes = 16 * W4 + 8;
    r->max_queue_mb = (double)w.max_wave * r->item_bytes / (1024.0 * 1024.0);
    r->time_to_bound_ms = w.t_ns / 1e6;
    r->engine = NR_ENGINE_WARP;
    r->stop = w.status;
    r->capacity = (uint64_t)cfg.pages * NR_PAGE;
}

// Solve n instances with the warp engine; instances the engine hands over
// (status 2) are left with engine = 0 for the caller.
static int ensure_host(void **buf, size_t *have, size_t need)
{
    if (*have >= need && *buf) return NR_OK;
    if (*buf) cudaFreeHost(*buf);
    *buf = nullptr;
    *have = 0;
    if (cudaMallocHost(buf, need) != cudaSuccess) {
        cudaGetLastError();
        *buf = nullptr;
        return NR_ERR_NOMEM;
    }
    *have = need;
    return NR_OK;
}

// Solve n instances with the warp engine; instances the engine hands over
// (status 2) are listed in *handover for the caller.  Host work per call:
// one layout pass, a parallel table fill into pinned staging memory, one
// upload, one launch per (group width, mask width) class, one download.
static int slot_ready(NrSlot &sl)
{
    if (sl.stream) return NR_OK;
    cudaError_t e = cudaStreamCreateWithFlags(&sl.stream, cudaStreamNonBlocking);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.ev0);
    if (e == cudaSuccess) e = cudaEventCreate(&sl.ev1);
    if (e != cudaSuccess) {
        nr_last_cuda_error(e, __FILE__, __LINE__, "batch stream set-up");
        return NR_ERR_CUDA;
    }
    return NR_OK;
}

// Order the work queued next on stream s after the work already queued on the
// caller's stream `after` (none: nothing to wait for).
static int wait_for_caller(nr_context *c, cudaStream_t s, cudaStream_t after)
{
    if (!after) return NR_OK;
    if (!c->ev_after) NR_CUDA_TRY(cudaEventCreateWithFlags(&c->ev_after, cudaEventDisableTiming));
    NR_CUDA_TRY(cudaEventRecord(c->ev_after, after));
    NR_CUDA_TRY(cudaStreamWaitEvent(s, c->ev_after, 0));
    return NR_OK;
}

// Kernel class of an instance: one lane per subproblem on undirected simple graphs (rows mode
// 1) of <= 16 nodes, and of <= 32 nodes in the two-slot kernel for breadth-first waves; else
// the lane-group kernel of its group width (8, 16, 32).  Each class is x the mask blocks.
static int small_class(const WarpRunCfg &cfg, bool lane_ok, int n, int rows, int w4)
{
    if (lane_ok && rows == 1 && n <= NR_LANE_MAX_N && w4 <= NR_LANE_MAX_W4) return NR_LANE_CLS0 + w4 - 1;
    if (lane_ok && rows == 1 && cfg.lane2 && cfg.lane_slots == 2 && n <= 32 && w4 <= NR_LANE32_MAX_W4)
        return NR_LANE32_CLS0 + w4 - 1;
    const int G = group_width(n);
    return (G == 8 ? 0 : G == 16 ? 1 : 2) * NR_MAX_W4 + w4 - 1;
}

// Build the tables of instances [0, n) of gs on the host and queue their
// upload, the kernels and the read-back of the outputs on slot `sl`.  `base`
// is the index of gs[0] in the caller's batch (for collected children).
static int warp_submit(nr_context *c, NrSlot &sl, int base, int n, const nr_graph *gs, const int32_t *srcs,
                       const int32_t *dsts, const WarpRunCfg &cfg, nr_result *res, PhaseClock &pc,
                       cudaStream_t after = nullptr, bool uniform = false, const double *pmat = nullptr)
{
    constexpr int NCLS = NR_NCLS;
    const bool lane_ok = cfg.lane && !cfg.fork && !cfg.learned && !cfg.dump && cfg.border != NR_BORDER_LEARNED;
    int rc0 = slot_ready(sl);
    if (rc0) return rc0;
    NrBatchScratch &S = sl.scratch;          // kept by the slot: no page faults on every call
    S.desc.resize(n);
    S.cls.resize(n);
    S.same_prev.resize(n);
    S.inst_b.resize(n);
    S.struct_b.resize(n);
    NrSmallGraph *desc = S.desc.data();
    // staging (the same offsets in pinned host memory and on the device):
    //   [work counters | tables (instance order) | descriptors (class order) | ids] then [outputs]
    size_t off_desc = 0, off_ids = 0, up_bytes = 0, off_out = 0;
    const size_t off_cnt = 0;
    int class_count[NCLS] = {0};
    int class_begin[NCLS + 1] = {0};
    unsigned char *hb = nullptr;
    NrSmallGraph *hdesc = nullptr;
    int *hids = nullptr;
    int rc = NR_OK;
    const int B = std::max(1, std::min(NR_HOST_BLOCKS, n / 128));
    auto blk_begin = [&](int b) { return (int)((long long)n * b / B); };
    if (pmat && !uniform) return NR_ERR_INVALID;
    if (uniform) {
        // one topology (the same CSR arrays) for every instance: every instance's tables have the
        // same size, so the offsets are known without a sizes pass -- instance 0's p, the shared
        // structural part, then the other instances' p -- and one parallel pass validates,
        // describes and copies them.  One class, so class order is instance order.
        int vr = validate_shape(&gs[0], srcs[0], dsts[0]);
        if (!vr) vr = validate_structure(&gs[0]);
        if (vr) return vr;
        NrSmallGraph t;
        const size_t ib = small_inst_layout(&gs[0], srcs[0], dsts[0], &t);
        const size_t sb = small_struct_layout(&gs[0], &t, 0);
        t.rows = rows_mode_of(&gs[0]);
        if (t.w4 > NR_MAX_W4) return NR_ERR_UNSUPPORTED;
        const int cls = small_class(cfg, lane_ok, gs[0].n_nodes, t.rows, t.w4);
        size_t off = align16(sizeof(int) * (NCLS + 1));   // work counters, then a NaN flag
        const size_t tbase = off;
        // matrix batches: the structural part, then the caller's matrix as it is (row i =
        // instance i's p; 8-byte rows suffice for the kernels' scalar loads)
        const size_t pm_row = sizeof(double) * (size_t)gs[0].n_edges;
        const size_t off_pm = pmat ? align16(tbase + sb) : 0;
        off = pmat ? align16(off_pm + (size_t)n * pm_row) : align16(off + (size_t)n * ib + sb);
        class_count[cls] = n;
        for (int j = 0; j < NCLS; ++j) class_begin[j + 1] = class_begin[j] + class_count[j];
        off_desc = off; off = align16(off + sizeof(NrSmallGraph) * n);
        off_ids = off; off = align16(off + sizeof(int) * n);
        up_bytes = off;
        off_out = off; off = align16(off + sizeof(NrWarpOut) * n);
        rc = ensure_host(&sl.hbuf, &sl.hbuf_bytes, off);
        if (rc) return rc;
        rc = ensure(&sl.wbuf, &sl.wbuf_bytes, off);
        if (rc) return rc;
        hb = static_cast<unsigned char *>(sl.hbuf);
        hdesc = reinterpret_cast<NrSmallGraph *>(hb + off_desc);
        hids = reinterpret_cast<int *>(hb + off_ids);
        memset(hb + off_cnt, 0, sizeof(int) * (NCLS + 1));
        t.struct_off = (long long)(pmat ? tbase : tbase + ib);
        small_fill_struct(&gs[0], &t, hb + t.struct_off);
        if (pmat) {
            // the matrix is the bulk of the upload: queue it, after the counters and the
            // structural part and before the descriptors are built, so that the copy runs while
            // the host writes them; then the scan of the matrix for NaN
            unsigned char *wb0 = static_cast<unsigned char *>(sl.wbuf);
            rc = wait_for_caller(c, sl.stream, after);
            if (rc) return rc;
            NR_CUDA_TRY(cudaMemcpyAsync(wb0, hb, off_pm, cudaMemcpyHostToDevice, sl.stream));
            NR_CUDA_TRY(cudaMemcpyAsync(wb0 + off_pm, pmat, (size_t)n * pm_row, cudaMemcpyHostToDevice, sl.stream));
            NR_CUDA_TRY(nr_launch_nan_scan(reinterpret_cast<const double *>(wb0 + off_pm), (size_t)n * gs[0].n_edges,
                                           reinterpret_cast<int *>(wb0 + sizeof(int) * NCLS), sl.stream));
        }
        pc.mark("sizes");
        std::atomic<int> bad(NR_OK);
        const int n_nodes0 = gs[0].n_nodes;
        c->parallel_for(B, 1, [&](int b) {
            for (int i = blk_begin(b), e = blk_begin(b + 1); i < e; ++i) {
                NrSmallGraph d = t;
                d.src = srcs[i];
                d.dst = dsts[i];
                if (pmat) {                   // terminals only: the matrix is uploaded as it is
                    if (d.src < 0 || d.dst < 0 || d.src >= n_nodes0 || d.dst >= n_nodes0) {
                        bad.store(NR_ERR_INVALID);
                        continue;
                    }
                    d.blob_off = (long long)(off_pm + (size_t)i * pm_row);
                    d.blob_bytes = (int)pm_row;
                } else {
                    const int v = validate_shape(&gs[i], srcs[i], dsts[i]);
                    if (v) { bad.store(v); continue; }
                    d.blob_off = (long long)(tbase + (i == 0 ? 0 : ib + sb + (size_t)(i - 1) * ib));
                    d.blob_bytes = (int)(ib + (i == 0 ? sb : 0));
                    if (!small_fill_inst(&gs[i], &d, hb + d.blob_off)) bad.store(NR_ERR_INVALID);
                }
                desc[i] = d;
                S.cls[i] = cls;
                hdesc[i] = d;
                hids[i] = i;
            }
        });
        if (bad.load() != NR_OK) return bad.load();
        sl.off_flag = sizeof(int) * NCLS;
        pc.mark("tables");
    } else {
    // Host blocks: contiguous instance ranges, one task of the worker pool each.  Two
    // parallel passes (sizes, then offsets and tables) around a serial prefix over blocks.
    S.blk.resize(B);
    std::atomic<int> too_wide(0), invalid(NR_OK);
    c->parallel_for(B, 1, [&](int b) {
        NrHostBlock &k = S.blk[b];
        size_t rel = 0;
        k.last_owner_rel = -1;
        k.last_rows = -1;
        for (int j = 0; j < NCLS; ++j) k.cnt[j] = 0;
        int cur_rows = -1;                    // rows mode of the current topology
        const int i0 = blk_begin(b);
        for (int i = i0, e = blk_begin(b + 1); i < e; ++i) {
            // validation (the shape of every instance; the arrays of the first of a run of
            // instances sharing them, and of the block's first, whose run may start earlier)
            int vr = validate_shape(&gs[i], srcs[i], dsts[i]);
            const bool prev_ok = i > 0 && validate_shape(&gs[i - 1], srcs[i - 1], dsts[i - 1]) == NR_OK;
            if (!vr && (i == i0 || !prev_ok || !same_structure_arrays(&gs[i], &gs[i - 1])))
                vr = validate_structure(&gs[i]);
            if (vr) { invalid.store(vr); S.cls[i] = 0; S.same_prev[i] = 0; S.inst_b[i] = 0; S.struct_b[i] = 0; continue; }
            // consecutive instances with the same topology share one structural part
            const bool same = prev_ok && same_topology(&gs[i], &gs[i - 1]);
            const size_t ib = small_inst_layout(&gs[i], srcs[i], dsts[i], &desc[i]);
            size_t sb = 0;                    // offsets relative to struct_off
            if (same && i > i0) {
                desc[i].off_eid = desc[i - 1].off_eid; desc[i].off_start = desc[i - 1].off_start;
                desc[i].off_list = desc[i - 1].off_list; desc[i].off_root_rows = desc[i - 1].off_root_rows;
            } else {
                sb = small_struct_layout(&gs[i], &desc[i], 0);
            }
            S.same_prev[i] = same;
            S.inst_b[i] = ib;
            S.struct_b[i] = same ? 0 : sb;
            rel += ib;
            if (!same) {
                k.last_owner_rel = (long long)rel;
                rel += sb;
                desc[i].rows = rows_mode_of(&gs[i]);
                k.last_rows = desc[i].rows;
                cur_rows = desc[i].rows;
            } else if (cur_rows < 0) {
                cur_rows = rows_mode_of(&gs[i]);   // its owner is in an earlier block
            }
            if (desc[i].w4 > NR_MAX_W4) { too_wide.store(1); S.cls[i] = 0; continue; }
            S.cls[i] = small_class(cfg, lane_ok, gs[i].n_nodes, cur_rows, desc[i].w4);
            k.cnt[S.cls[i]]++;
        }
        k.bytes = rel;
    });
    if (invalid.load() != NR_OK) return invalid.load();
    if (too_wide.load()) return NR_ERR_UNSUPPORTED;
    pc.mark("sizes");

    size_t off = align16(sizeof(int) * NCLS);
    long long owner_struct = -1;              // struct_off of the last structural part so far
    int owner_rows = 0;                       // and its rows mode
    for (int b = 0; b < B; ++b) {
        NrHostBlock &k = S.blk[b];
        k.base = off;
        k.struct_in = owner_struct;
        k.rows_in = owner_rows;
        if (k.last_owner_rel >= 0) owner_struct = (long long)off + k.last_owner_rel;
        if (k.last_rows >= 0) owner_rows = k.last_rows;
        off += k.bytes;
        for (int j = 0; j < NCLS; ++j) {
            k.cbase[j] = class_count[j];
            class_count[j] += k.cnt[j];
        }
    }
    for (int j = 0; j < NCLS; ++j) class_begin[j + 1] = class_begin[j] + class_count[j];
    off = align16(off);
    off_desc = off; off = align16(off + sizeof(NrSmallGraph) * n);
    off_ids = off; off = align16(off + sizeof(int) * n);
    up_bytes = off;
    off_out = off; off = align16(off + sizeof(NrWarpOut) * n);
    rc = ensure_host(&sl.hbuf, &sl.hbuf_bytes, off);
    if (rc) return rc;
    rc = ensure(&sl.wbuf, &sl.wbuf_bytes, off);
    if (rc) return rc;
    hb = static_cast<unsigned char *>(sl.hbuf);
    hdesc = reinterpret_cast<NrSmallGraph *>(hb + off_desc);
    hids = reinterpret_cast<int *>(hb + off_ids);
    memset(hb + off_cnt, 0, sizeof(int) * NCLS);
    std::atomic<int> bad_p(0);            // a NaN probability
    c->parallel_for(B, 1, [&](int b) {
        const NrHostBlock &k = S.blk[b];
        size_t at = k.base;
        long long rep = k.struct_in;
        int rep_rows = k.rows_in;
        int fill[NCLS];
        for (int j = 0; j < NCLS; ++j) fill[j] = class_begin[j] + k.cbase[j];
        for (int i = blk_begin(b), e = blk_begin(b + 1); i < e; ++i) {
            NrSmallGraph &d = desc[i];
            d.blob_off = (long long)at;
            at += S.inst_b[i];
            if (!S.same_prev[i]) {
                d.struct_off = (long long)at;
                rep = d.struct_off;
                rep_rows = d.rows;
                at += S.struct_b[i];
                small_fill_struct(&gs[i], &d, hb + d.struct_off);
            } else {
                d.struct_off = rep;               // instance 0 always owns one, so rep >= 0 here
                d.rows = rep_rows;
            }
            d.blob_bytes = (int)(S.inst_b[i] + S.struct_b[i]);
            if (!small_fill_inst(&gs[i], &d, hb + d.blob_off)) bad_p.store(1);
            const int slot = fill[S.cls[i]]++;
            hdesc[slot] = d;
            hids[slot] = i;
        }
    });
    if (bad_p.load()) return NR_ERR_INVALID;
    pc.mark("tables");
    }

    // launch geometry per class (occupancy cached per kernel and shared-memory size)
    const int warps_pb = cfg.warps_per_block, block = 32 * warps_pb;
    if (!c->smem_optin) {
        int v = 0;
        NR_CUDA_TRY(cudaDeviceGetAttribute(&v, cudaDevAttrMaxSharedMemoryPerBlockOptin, c->device));
        c->smem_optin = v;
    }
    // pages per warp: as asked, but no more than the block's shared memory can index
    WarpRunCfg cfgp = cfg;
    while (cfgp.pages > 4 &&
           std::max(std::max(nr_warp_shm_bytes(4, NR_MAX_W4, cfgp.n_buckets, cfgp.pages, true),
                             nr_lane_shm_bytes(cfgp.n_buckets, cfgp.pages)),
                    nr_lane2_shm_bytes(cfgp.pages, cfg.lane_slots)) * warps_pb > (size_t)c->smem_optin)
        cfgp.pages /= 2;
    const bool learn = cfg.learned || cfg.dump || cfg.border == NR_BORDER_LEARNED;
    int grids[NCLS] = {0}, wpbs[NCLS] = {0}, nps[NCLS] = {0};
    size_t smems[NCLS] = {0};
    size_t slab_need = 0;
    for (int j = 0; j < NCLS; ++j) {
        if (!class_count[j]) continue;
        const bool lanek = j >= NR_LANE_CLS0, lane32 = j >= NR_LANE32_CLS0;
        const int G = lanek ? 0 : 8 << (j / NR_MAX_W4);
        const int W4 = lane32 ? j - NR_LANE32_CLS0 + 1 : lanek ? j - NR_LANE_CLS0 + 1 : j % NR_MAX_W4 + 1;
        const bool two = lanek && cfg.lane2;
        const int slots = lane32 ? 2 : cfg.lane_slots, rb = lane32 ? 32 : 16;
        // the 32-bit-row kernel's warps hold a pool of two slots' worth: each slot (instance) gets
        // the pages one instance has in the lane-group kernel it stands in for; its blocks have as
        // many of the asked warps as their shared memory holds
        int np = lane32 ? 2 * cfgp.pages : cfgp.pages, wpb = warps_pb;
        if (lane32) {
            while (wpb > 1 && nr_lane2_shm_bytes(np, 2, 32) * wpb > (size_t)c->smem_optin) --wpb;
            while (np > 8 && nr_lane2_shm_bytes(np, 2, 32) > (size_t)c->smem_optin) np /= 2;
        }
        const void *kfn = lanek ? (two ? nr_lane2_kernel_ptr(W4, slots, rb) : nr_lane_kernel_ptr(W4))
                                : warp_kernel(G, W4, learn, cfg.fork != 0);
        if (!kfn) return NR_ERR_UNSUPPORTED;
        const size_t smem = (two ? nr_lane2_shm_bytes(np, slots, rb)
                                 : lanek ? nr_lane_shm_bytes(cfg.n_buckets, cfgp.pages)
                                         : nr_warp_shm_bytes(32 / G, W4, cfg.n_buckets, cfgp.pages, learn)) * wpb;
        auto it = c->occupancy.find({kfn, smem * 64 + wpb});
        int bps;
        if (it == c->occupancy.end()) {
            NR_CUDA_TRY(nr_smem_limit(c->device, kfn, smem));
            NR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, kfn, 32 * wpb, smem));
            c->occupancy[{kfn, smem * 64 + wpb}] = bps;
        } else {
            bps = it->second;
        }
        if (bps < 1) return NR_ERR_UNSUPPORTED;
        const int per_block = wpb * (two ? slots : 1);   // instances a block starts with
        grids[j] = std::max(1, std::min(bps * c->sms, (class_count[j] + per_block - 1) / per_block));
        smems[j] = smem;
        wpbs[j] = wpb;
        nps[j] = np;
        const size_t row_bytes = lane32 ? 128 : lanek ? 4 * (size_t)NR_LANE_ROW_WORDS : 4 * (size_t)G;
        slab_need = std::max(slab_need, (size_t)grids[j] * wpb * np * NR_PAGE *
                                            (16 * (size_t)W4 + 8 + row_bytes));
    }
    rc = ensure(&sl.wslab, &sl.wslab_bytes, slab_need);
    if (rc) return rc;
    unsigned char *wb = static_cast<unsigned char *>(sl.wbuf);
    cudaStream_t s = sl.stream;
    pc.mark("geometry");
    if (pmat) {
        // counters, structural part and the caller's matrix (straight from its memory: a plain
        // DMA when it is pinned) are queued already, with the NaN scan; descriptors and ids now
        NR_CUDA_TRY(cudaMemcpyAsync(wb + off_desc, hb + off_desc, up_bytes - off_desc, cudaMemcpyHostToDevice, s));
    } else {
        rc = wait_for_caller(c, s, after);
        if (rc) return rc;
        NR_CUDA_TRY(cudaMemcpyAsync(wb, hb, up_bytes, cudaMemcpyHostToDevice, s));
    }
    NR_CUDA_TRY(cudaEventRecord(sl.ev0, s));
    int first_grid = 0;
    for (int j = 0; j < NCLS; ++j) {
        if (!class_count[j]) continue;
        const bool lanek = j >= NR_LANE_CLS0, lane32 = j >= NR_LANE32_CLS0;
        const int G = lanek ? 0 : 8 << (j / NR_MAX_W4);
        const int W4 = lane32 ? j - NR_LANE32_CLS0 + 1 : lanek ? j - NR_LANE_CLS0 + 1 : j % NR_MAX_W4 + 1;
        if (!first_grid) first_grid = grids[j];
        const int np = nps[j], wpb = wpbs[j];     // pages a warp holds, warps a block (see above)
        NrWarpParams P;
        P.blob = wb;
        P.inst = reinterpret_cast<const NrSmallGraph *>(wb + off_desc) + class_begin[j];
        P.inst_id = reinterpret_cast<const int *>(wb + off_ids) + class_begin[j];
        P.n_inst = class_count[j];
        P.next_inst = reinterpret_cast<int *>(wb + off_cnt) + j;
        P.slab_mask = static_cast<uint4 *>(sl.wslab);
        const size_t warps = (size_t)grids[j] * wpb;
        P.slab_mass = reinterpret_cast<double *>(static_cast<unsigned char *>(sl.wslab) +
                                                 warps * np * NR_PAGE * 16 * (size_t)W4);
        P.slab_rows = reinterpret_cast<uint32_t *>(static_cast<unsigned char *>(sl.wslab) +
                                                   warps * np * NR_PAGE * (16 * (size_t)W4 + 8));
        P.pages = np;
        P.n_buckets = cfg.n_buckets;
        P.shift = cfg.shift;
        P.wave_mode = cfg.wave_mode;
        P.escalate = cfg.escalate;
        P.eps = cfg.eps;
        P.target = cfg.target;
        P.target_fix = nr_fix_of(cfg.target);
        P.max_nodes = cfg.max_nodes;
        P.out = reinterpret_cast<NrWarpOut *>(wb + off_out);
        P.learned = cfg.learned;
        P.mlp = c->mlp;
        P.dump_feat = cfg.dump ? cfg.dump->feat : nullptr;
        P.dump_mask = cfg.dump ? cfg.dump->mask : nullptr;
        P.dump_mass = cfg.dump ? cfg.dump->mass : nullptr;
        P.dump_inst = cfg.dump ? cfg.dump->inst : nullptr;
        P.dump_count = cfg.dump ? cfg.dump->count : nullptr;
        P.dump_cap = cfg.dump ? cfg.dump->cap : 0;
        P.dump_stride = cfg.dump ? cfg.dump->stride : 0;
        P.inst_base = base;
        P.fork = cfg.fork;
        P.step_cap = cfg.step_cap;
        P.border = cfg.border;
        P.handover_pages = (lanek && cfg.lane2) ? cfg.handover_pages : 0;
        const void *kfn = lanek ? (cfg.lane2 ? nr_lane2_kernel_ptr(W4, lane32 ? 2 : cfg.lane_slots, lane32 ? 32 : 16)
                                             : nr_lane_kernel_ptr(W4))
                                : warp_kernel(G, W4, learn, cfg.fork != 0);
        void *args[] = {&P};
        NR_CUDA_TRY(nr_smem_limit(c->device, kfn, smems[j]));
        NR_CUDA_TRY(cudaLaunchKernel(kfn, dim3(grids[j]), dim3(32 * wpb), args, smems[j], s));
    }
    NR_CUDA_TRY(cudaEventRecord(sl.ev1, s));
    NrWarpOut *hout = reinterpret_cast<NrWarpOut *>(hb + off_out);
    NR_CUDA_TRY(cudaMemcpyAsync(hout, wb + off_out, sizeof(NrWarpOut) * n, cudaMemcpyDeviceToHost, s));
    if (pmat) NR_CUDA_TRY(cudaMemcpyAsync(hb + sl.off_flag, wb + sl.off_flag, sizeof(int), cudaMemcpyDeviceToHost, s));
    sl.matrix = (pmat != nullptr);
    sl.pmat = pmat;
    sl.n = n; sl.gs = gs; sl.srcs = srcs; sl.dsts = dsts; sl.res = res;
    sl.cfgp = cfgp; sl.off_out = off_out; sl.first_grid = first_grid; sl.block = block;
    for (int j = 0; j < NCLS; ++j) sl.nps[j] = nps[j];
    pc.mark("enqueue");
    return NR_OK;
}

// Instances the two-slot lane kernel handed over (status 2 in breadth-first waves: a next wave
// above cfg.handover_pages pages) run again from their roots on the block kernel, a block each,
// from the slot's tables (still on the device); each gets wave buffers of the pages its slot
// could hold.  ids: the part's indices.  Fills their results; *ms = the launches' device time.
static int block_handover(nr_context *c, NrSlot &sl, const std::vector<int> &ids, float *ms)
{
    const NrSmallGraph *desc = sl.scratch.desc.data();
    const std::vector<int> &cls = sl.scratch.cls;
    const int k = (int)ids.size();
    // grouped by kernel class; in a class the largest next wave at the hand-over first, so the
    // largest instances do not start last and leave the launch with a tail
    const NrWarpOut *lout = reinterpret_cast<const NrWarpOut *>(static_cast<unsigned char *>(sl.hbuf) + sl.off_out);
    std::vector<int> order(ids);
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return cls[a] != cls[b] ? cls[a] < cls[b] : lout[a].queued > lout[b].queued;
    });
    // staging: [work counters | descriptors | ids] then [outputs]
    const size_t off_desc = align16(sizeof(int) * NR_NCLS);
    const size_t off_ids = align16(off_desc + sizeof(NrSmallGraph) * k);
    const size_t off_out = align16(off_ids + sizeof(int) * k);
    const size_t bytes = align16(off_out + sizeof(NrWarpOut) * k);
    int rc = ensure_host(&sl.hv_host, &sl.hv_host_bytes, bytes);
    if (!rc) rc = ensure(&sl.hv_dev, &sl.hv_dev_bytes, bytes);
    if (rc) return rc;
    unsigned char *hb = static_cast<unsigned char *>(sl.hv_host), *db = static_cast<unsigned char *>(sl.hv_dev);
    memset(hb, 0, off_desc);
    NrSmallGraph *hd = reinterpret_cast<NrSmallGraph *>(hb + off_desc);
    int *hid = reinterpret_cast<int *>(hb + off_ids);
    for (int j = 0; j < k; ++j) { hd[j] = desc[order[j]]; hid[j] = j; }
    const WarpRunCfg &cfg = sl.cfgp;
    // launch geometry per class; the classes run side by side (up to NR_HV_STREAMS streams, the
    // most work first), each in its own part of the slab, so a small class fills the large one's tail
    struct Grp { int j0, j1, w4, rb, grid, budget; const void *kfn; size_t smem, slab_off, work; };
    std::vector<Grp> grps;
    size_t slab_need = 0;
    for (int j0 = 0; j0 < k;) {
        const int cj = cls[order[j0]];
        int j1 = j0;
        while (j1 < k && cls[order[j1]] == cj) ++j1;
        if (cj < NR_LANE_CLS0) return NR_ERR_INTERNAL;       // only lane kernels hand over here
        const bool lane32 = cj >= NR_LANE32_CLS0;
        Grp gr;
        gr.j0 = j0; gr.j1 = j1;
        gr.w4 = lane32 ? cj - NR_LANE32_CLS0 + 1 : cj - NR_LANE_CLS0 + 1;
        gr.rb = lane32 ? 32 : 16;
        gr.kfn = nr_block_lane_kernel_ptr(gr.w4, gr.rb);
        if (!gr.kfn) return NR_ERR_INTERNAL;
        gr.smem = nr_block_lane_shm_bytes(gr.rb);
        auto it = c->occupancy.find({gr.kfn, gr.smem * 64 + NR_BLOCK_LANE_WARPS});
        int bps;
        if (it == c->occupancy.end()) {
            NR_CUDA_TRY(nr_smem_limit(c->device, gr.kfn, gr.smem));
            NR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, gr.kfn, NR_BLOCK_LANE_THREADS, gr.smem));
            c->occupancy[{gr.kfn, gr.smem * 64 + NR_BLOCK_LANE_WARPS}] = bps;
        } else {
            bps = it->second;
        }
        if (bps < 1) return NR_ERR_UNSUPPORTED;
        gr.grid = std::max(1, std::min(j1 - j0, bps * c->sms));
        gr.budget = std::max(1, sl.nps[cj] / (lane32 ? 2 : cfg.lane_slots));   // pages one slot may hold
        gr.slab_off = slab_need;
        slab_need += align16((size_t)gr.grid * 2 * gr.budget * NR_PAGE * nr_block_lane_rec_bytes(gr.w4, gr.rb));
        gr.work = 0;
        for (int j = j0; j < j1; ++j) gr.work += lout[order[j]].queued;
        grps.push_back(gr);
        j0 = j1;
    }
    std::stable_sort(grps.begin(), grps.end(), [](const Grp &a, const Grp &b) { return a.work > b.work; });
    rc = ensure(&sl.wslab, &sl.wslab_bytes, slab_need);
    if (rc) return rc;
    cudaStream_t s = sl.stream;
    const int nside = std::min<int>(NR_HV_STREAMS, (int)grps.size());
    if (nside > 1) {
        if (!sl.hv_fork) NR_CUDA_TRY(cudaEventCreateWithFlags(&sl.hv_fork, cudaEventDisableTiming));
        for (int q = 0; q < nside; ++q) {
            if (!sl.hv_side[q]) NR_CUDA_TRY(cudaStreamCreateWithFlags(&sl.hv_side[q], cudaStreamNonBlocking));
            if (!sl.hv_join[q]) NR_CUDA_TRY(cudaEventCreateWithFlags(&sl.hv_join[q], cudaEventDisableTiming));
        }
    }
    NR_CUDA_TRY(cudaMemcpyAsync(db, hb, off_out, cudaMemcpyHostToDevice, s));
    NR_CUDA_TRY(cudaEventRecord(sl.ev0, s));
    if (nside > 1) {
        NR_CUDA_TRY(cudaEventRecord(sl.hv_fork, s));
        for (int q = 0; q < nside; ++q) NR_CUDA_TRY(cudaStreamWaitEvent(sl.hv_side[q], sl.hv_fork, 0));
    }
    for (size_t gi = 0; gi < grps.size(); ++gi) {
        const Grp &gr = grps[gi];
        const size_t cap = (size_t)gr.budget * NR_PAGE;
        unsigned char *slab = static_cast<unsigned char *>(sl.wslab) + gr.slab_off;
        cudaStream_t gs_ = nside > 1 ? sl.hv_side[gi % nside] : s;
        NrWarpParams P{};
        P.blob = static_cast<const unsigned char *>(sl.wbuf);
        P.inst = reinterpret_cast<const NrSmallGraph *>(db + off_desc) + gr.j0;
        P.inst_id = reinterpret_cast<const int *>(db + off_ids) + gr.j0;
        P.n_inst = gr.j1 - gr.j0;
        P.next_inst = reinterpret_cast<int *>(db) + cls[order[gr.j0]];
        P.slab_mask = reinterpret_cast<uint4 *>(slab);
        P.slab_mass = reinterpret_cast<double *>(slab + (size_t)gr.grid * 2 * cap * 16 * gr.w4);
        P.slab_rows = reinterpret_cast<uint32_t *>(slab + (size_t)gr.grid * 2 * cap * (16 * gr.w4 + 8));
        P.pages = gr.budget;
        P.n_buckets = cfg.n_buckets;
        P.shift = -1;
        P.wave_mode = 1;
        P.eps = cfg.eps;
        P.target = cfg.target;
        P.target_fix = nr_fix_of(cfg.target);
        P.max_nodes = cfg.max_nodes;
        P.out = reinterpret_cast<NrWarpOut *>(db + off_out);
        P.step_cap = cfg.step_cap;
        P.border = cfg.border;
        void *args[] = {&P};
        NR_CUDA_TRY(nr_smem_limit(c->device, gr.kfn, gr.smem));
        NR_CUDA_TRY(cudaLaunchKernel(gr.kfn, dim3(gr.grid), dim3(NR_BLOCK_LANE_THREADS), args, gr.smem, gs_));
    }
    if (nside > 1)
        for (int q = 0; q < nside; ++q) {
            NR_CUDA_TRY(cudaEventRecord(sl.hv_join[q], sl.hv_side[q]));
            NR_CUDA_TRY(cudaStreamWaitEvent(s, sl.hv_join[q], 0));
        }
    NR_CUDA_TRY(cudaEventRecord(sl.ev1, s));
    const NrWarpOut *hout = reinterpret_cast<const NrWarpOut *>(hb + off_out);
    NR_CUDA_TRY(cudaMemcpyAsync(hb + off_out, db + off_out, sizeof(NrWarpOut) * k, cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaStreamSynchronize(s));
    NR_CUDA_TRY(cudaEventElapsedTime(ms, sl.ev0, sl.ev1));
    for (const Grp &gr : grps)
        for (int j = gr.j0; j < gr.j1; ++j) {
            const int i = order[j];
            if (hout[j].status == NR_LANE_STATUS_CHECK) {
                snprintf(g_internal, sizeof(g_internal), "block kernel check %llu failed on instance %d",
                         (unsigned long long)hout[j].max_wave, i);
                return NR_ERR_INTERNAL;
            }
            nr_result *r = &sl.res[i];
            fill_from_warp(hout[j], cfg, desc[i].w4, r);
            r->kernel = NR_KERNEL_BLOCK;
            r->capacity = (uint64_t)gr.budget * NR_PAGE;
            r->grid_blocks = gr.grid;
            r->block_threads = NR_BLOCK_LANE_THREADS;
            r->h2d_bytes = desc[i].blob_bytes + 2 * sizeof(NrSmallGraph) + 2 * sizeof(int);
            r->d2h_bytes = 2 * sizeof(NrWarpOut);
        }
    return NR_OK;
}

// Wait for the part queued on slot `sl` and fill its results; instances the
// warp engine handed over are appended to `handover` (plus `base`).
static int warp_finish(nr_context *c, NrSlot &sl, int base, std::vector<int> *handover, PhaseClock &pc)
{
    NR_CUDA_TRY(cudaStreamSynchronize(sl.stream));
    pc.mark("device");
    float ms = 0.f;
    NR_CUDA_TRY(cudaEventElapsedTime(&ms, sl.ev0, sl.ev1));
    const int n = sl.n;
    const nr_graph *gs = sl.gs;
    const NrSmallGraph *desc = sl.scratch.desc.data();
    const NrWarpOut *hout = reinterpret_cast<const NrWarpOut *>(static_cast<unsigned char *>(sl.hbuf) + sl.off_out);
    if (sl.matrix && *reinterpret_cast<const int *>(static_cast<unsigned char *>(sl.hbuf) + sl.off_flag))
        return NR_ERR_INVALID;                // a NaN probability in the caller's matrix
    const int gstride = sl.matrix ? 0 : 1;    // matrix batches: one topology for every instance
    std::atomic<int> n_hand(0), n_check(0);
    c->parallel_for(n, 256, [&](int i) {
        nr_result *r = &sl.res[i];
        memset(r, 0, sizeof(*r));
        const nr_graph &gi = gs[i * gstride];
        r->n_nodes = gi.n_nodes; r->n_edges = gi.n_edges; r->src = sl.srcs[i]; r->dst = sl.dsts[i];
        r->mask_words = std::max(1, (2 * gi.n_edges + 31) / 32);
        if (hout[i].status == 2) { n_hand.fetch_add(1); return; }
        if (hout[i].status == NR_LANE_STATUS_CHECK) { n_check.fetch_add(1); return; }
        fill_from_warp(hout[i], sl.cfgp, desc[i].w4, r);
        r->kernel = sl.scratch.cls[i] < NR_LANE_CLS0 ? NR_KERNEL_GROUP
                    : sl.cfgp.lane2 ? NR_KERNEL_LANE2 : NR_KERNEL_LANE;
        r->ms = ms;
        r->grid_blocks = sl.first_grid;
        r->block_threads = sl.block;
        r->h2d_bytes = desc[i].blob_bytes + sizeof(NrSmallGraph) + sizeof(int);
        r->d2h_bytes = sizeof(NrWarpOut);
    });
    if (n_check.load()) {
        for (int i = 0; i < n; ++i)
            if (hout[i].status == NR_LANE_STATUS_CHECK) {
                snprintf(g_internal, sizeof(g_internal), "warp engine check %llu failed on instance %d",
                         (unsigned long long)hout[i].max_wave, base + i);
                break;
            }
        return NR_ERR_INTERNAL;
    }
    if (n_hand.load()) {
        // breadth-first waves: the two-slot lane kernel's hand-overs run on the block kernel now;
        // the others (exhaustive runs past a warp's budget) on the whole-GPU engine after the part
        std::vector<int> blk;
        for (int i = 0; i < n; ++i)
            if (hout[i].status == 2) {
                if (sl.cfgp.wave_mode && sl.cfgp.lane2 && sl.scratch.cls[i] >= NR_LANE_CLS0) blk.push_back(i);
                else handover->push_back(base + i);
            }
        if (!blk.empty()) {
            float ms2 = 0.f;
            const int rc = block_handover(c, sl, blk, &ms2);
            if (rc) return rc;
            for (int i = 0; i < n; ++i) sl.res[i].ms = ms + ms2;   // the part's device time
        }
    }
    pc.mark("results");
    return NR_OK;
}

// Warp engine over instances [0, n) on slot 0.
int run_warp_batch(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                          const WarpRunCfg &cfg, nr_result *res, std::vector<int> *handover,
                          PhaseClock *clock)
{
    PhaseClock local;
    PhaseClock &pc = clock ? *clock : local;
    int rc = warp_submit(c, c->slot[0], 0, n, gs, srcs, dsts, cfg, res, pc);
    if (rc) return rc;
    return warp_finish(c, c->slot[0], 0, handover, pc);
}

// Checks of a batch: shapes, CSR arrays (once per run of instances sharing them),
// probabilities of graphs above 32 nodes (the warp engine checks its own while
// copying them).  *n_wide = graphs above 32 nodes.
// The branch order: a known value; the learned one needs a model and runs on the warp engine
// only (a target width or a max-mass / learned order, path branching).
int branch_order_ok(const nr_context *c, const nr_options &o)
{
    if (o.branch_order < NR_BORDER_SRC || o.branch_order > NR_BORDER_LEARNED) return NR_ERR_INVALID;
    if (o.branch_order != NR_BORDER_LEARNED) return NR_OK;
    if (!c->has_model) return NR_ERR_INVALID;
    if (o.branching != NR_BRANCH_PATH) return NR_ERR_UNSUPPORTED;
    if (!(o.target_width > 0) && o.order != NR_ORDER_MAXMASS && o.order != NR_ORDER_LEARNED) return NR_ERR_UNSUPPORTED;
    return NR_OK;
}

static int batch_options_ok(const nr_context *c, const nr_options &o)
{
    if (o.order == NR_ORDER_LEARNED && !c->has_model) return NR_ERR_INVALID;
    if (const int rb = branch_order_ok(c, o)) return rb;
    if (o.order == NR_ORDER_LEARNED && o.branching == NR_BRANCH_FORK) return NR_ERR_UNSUPPORTED;
    if (o.branching != NR_BRANCH_PATH && o.branching != NR_BRANCH_FORK) return NR_ERR_INVALID;
    return NR_OK;
}

static int batch_validate(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                          const nr_options &o, int *n_wide)
{
    std::atomic<int> bad(NR_OK), wide(0);
    c->parallel_for(n, 256, [&](int i) {
        int rc = validate_shape(&gs[i], srcs[i], dsts[i]);
        if (!rc && !(i > 0 && same_structure_arrays(&gs[i], &gs[i - 1]))) rc = validate_structure(&gs[i]);
        if (!rc && gs[i].n_nodes > NR_SMALL_MAX_N) {
            rc = validate_probabilities(&gs[i]);
            // the learned queue order: n <= 32 only; the learned branch order: in the bucketed
            // whole-GPU queue (max-mass order) only
            const bool buckets = o.bucket_shift >= 0 &&
                                 (o.order == NR_ORDER_MAXMASS || (o.order == NR_ORDER_AUTO && o.target_width > 0));
            if (!rc && (o.order == NR_ORDER_LEARNED || (o.branch_order == NR_BORDER_LEARNED && !buckets)))
                rc = NR_ERR_UNSUPPORTED;
            wide.fetch_add(1);
        }
        if (rc) bad.store(rc);
    });
    *n_wide = wide.load();
    if (bad.load() != NR_OK) return bad.load();
    return batch_options_ok(c, o);
}

static WarpRunCfg batch_cfg(const nr_options &o, uint64_t capacity)
{
    const bool exhaustive = !(o.target_width > 0) && o.order != NR_ORDER_MAXMASS && o.order != NR_ORDER_LEARNED;
    return warp_cfg(&o, capacity, exhaustive);
}

// Instances the warp engine handed over (exhaustive runs that outgrew a warp's
// budget) finish on the whole-GPU engine.
static int run_handover(nr_context *c, const std::vector<int> &handover, const nr_graph *gs, const int32_t *srcs,
                        const int32_t *dsts, uint64_t capacity, const nr_options &o, nr_result *res,
                        const double *pmat = nullptr)
{
    for (int i : handover) {
        nr_graph gi = pmat ? gs[0] : gs[i];      // matrix batches: the topology with row i of the matrix
        if (pmat) gi.edge_p = pmat + (size_t)i * gi.n_edges;
        const int rc = run_grid_small(c, &gi, srcs[i], dsts[i], std::max<uint64_t>(capacity, 1u << 22), &o, &res[i]);
        if (rc) return rc;
    }
    return NR_OK;
}

// ---------------------------------------------------------------------------
// graphs of 33..64 nodes on the 64-bit-row block kernel (nr_block64.cuh)
// ---------------------------------------------------------------------------

// An undirected simple graph of 33..64 nodes and <= 256 edges: every edge id on exactly the
// arcs u -> v and v -> u, no self-loop, no ordered pair twice.
static bool mid_ok(const nr_graph &g)
{
    const int n = g.n_nodes, E = g.n_edges;
    if (n <= NR_SMALL_MAX_N || n > NR_MID_MAX_N || E > NR_MID_MAX_E || g.n_arcs != 2 * E) return false;
    static thread_local int pid[NR_MID_MAX_N][NR_MID_MAX_N];
    for (int u = 0; u < n; ++u)
        for (int v = 0; v < n; ++v) pid[u][v] = -1;
    std::vector<int> cnt(std::max(E, 1), 0);
    for (int u = 0; u < n; ++u)
        for (int j = g.row_ptr[u]; j < g.row_ptr[u + 1]; ++j) {
            const int v = g.col_idx[j], e = g.edge_id[j];
            if (v == u || pid[u][v] != -1) return false;
            pid[u][v] = e;
            cnt[e]++;
        }
    for (int e = 0; e < E; ++e)
        if (cnt[e] != 2) return false;
    for (int u = 0; u < n; ++u)
        for (int j = g.row_ptr[u]; j < g.row_ptr[u + 1]; ++j)
            if (pid[g.col_idx[j]][u] != g.edge_id[j]) return false;
    return true;
}

// One instance's tables: [p: E doubles][endpoints: E x u16, u | v << 8][edge ids: 64 x 64 u16].
static size_t mid_layout(const nr_graph &g, int src, int dst, NrSmallGraph *sg)
{
    memset(sg, 0, sizeof(*sg));
    const int E = g.n_edges, W = std::max(1, (2 * E + 31) / 32);
    sg->n = g.n_nodes; sg->e = E; sg->w4 = (W + 3) / 4; sg->src = src; sg->dst = dst;
    sg->n_in = g.n_arcs;
    sg->rows = 1;
    size_t off = 0;
    sg->off_p = 0; off = align16(sizeof(double) * std::max(E, 1));
    sg->off_list = (int)off; off = align16(off + sizeof(uint16_t) * std::max(E, 1));
    sg->off_eid = (int)off; off = align16(off + sizeof(uint16_t) * NR_MID_MAX_N * NR_MID_MAX_N);
    sg->blob_bytes = (int)off;
    return off;
}

static void mid_fill(const nr_graph &g, const NrSmallGraph &sg, unsigned char *b)
{
    memcpy(b + sg.off_p, g.edge_p, sizeof(double) * g.n_edges);
    uint16_t *ends = reinterpret_cast<uint16_t *>(b + sg.off_list);
    uint16_t *eid = reinterpret_cast<uint16_t *>(b + sg.off_eid);
    for (int i = 0; i < NR_MID_MAX_N * NR_MID_MAX_N; ++i) eid[i] = 0xffff;
    for (int u = 0; u < g.n_nodes; ++u)
        for (int j = g.row_ptr[u]; j < g.row_ptr[u + 1]; ++j) {
            const int v = g.col_idx[j], e = g.edge_id[j];
            eid[u * NR_MID_MAX_N + v] = (uint16_t)e;
            if (u < v) ends[e] = (uint16_t)(u | (v << 8));
        }
}

// The graphs idx (mid_ok) in breadth-first waves, one block each: tables to the control buffer,
// wave buffers of `cap` records per block in the arena, one launch per mask width.
static int run_block64(nr_context *c, const std::vector<int> &idx, const nr_graph *gs, const int32_t *srcs,
                       const int32_t *dsts, uint64_t cap, const WarpRunCfg &cfg, nr_result *res)
{
    c->ckpt.valid = false;                 // the arena is about to be reused
    const int k = (int)idx.size();
    std::vector<NrSmallGraph> d(k);
    size_t blob = 0;
    for (int j = 0; j < k; ++j) {
        const int i = idx[j];
        const size_t b = mid_layout(gs[i], srcs[i], dsts[i], &d[j]);
        d[j].blob_off = d[j].struct_off = (long long)blob;
        blob += b;
        if (d[j].w4 > NR_MID_MAX_W4) return NR_ERR_INTERNAL;
    }
    // one launch per mask width; inside it the largest graphs first
    std::vector<int> order(k);
    for (int j = 0; j < k; ++j) order[j] = j;
    std::stable_sort(order.begin(), order.end(), [&](int a, int b) {
        return d[a].w4 != d[b].w4 ? d[a].w4 < d[b].w4 : d[a].e > d[b].e;
    });
    const size_t off_blob = 16;
    const size_t off_desc = align16(off_blob + blob);
    const size_t off_ids = align16(off_desc + sizeof(NrSmallGraph) * k);
    const size_t off_out = align16(off_ids + sizeof(int) * k);
    const size_t total = align16(off_out + sizeof(NrWarpOut) * k);
    int rc = ensure(&c->sbuf, &c->sbytes, total);
    if (rc) return rc;
    std::vector<unsigned char> up(off_out, 0);
    NrSmallGraph *hd = reinterpret_cast<NrSmallGraph *>(up.data() + off_desc);
    int *hid = reinterpret_cast<int *>(up.data() + off_ids);
    for (int j = 0; j < k; ++j) {
        NrSmallGraph t = d[order[j]];
        mid_fill(gs[idx[order[j]]], t, up.data() + off_blob + t.blob_off);
        t.blob_off += (long long)off_blob;
        t.struct_off = t.blob_off;
        hd[j] = t;
        hid[j] = j;
    }
    unsigned char *sb = static_cast<unsigned char *>(c->sbuf);
    cudaStream_t s = c->stream;
    NR_CUDA_TRY(cudaMemcpyAsync(sb, up.data(), off_out, cudaMemcpyHostToDevice, s));
    const int optin = smem_optin(c);
    const int pages = (int)std::max<uint64_t>(1, std::min<uint64_t>(cap / NR_PAGE, 1u << 30));
    const size_t capr = (size_t)pages * NR_PAGE;
    struct Grp { int j0, j1, w4, warps, grid; size_t smem; int row_words; const void *kfn; };
    std::vector<Grp> grps;
    size_t slab_need = 0;
    size_t free_b = 0, total_b = 0;
    NR_CUDA_TRY(cudaMemGetInfo(&free_b, &total_b));
    for (int j0 = 0; j0 < k;) {
        Grp gr;
        gr.j0 = j0;
        gr.w4 = hd[j0].w4;
        int j1 = j0, nmax = 1;
        while (j1 < k && hd[j1].w4 == gr.w4) nmax = std::max(nmax, hd[j1++].n);
        gr.j1 = j1;
        gr.row_words = 2 * nmax;
        gr.kfn = nr_block64_kernel_ptr(gr.w4);
        if (!gr.kfn) return NR_ERR_INTERNAL;
        const size_t per_warp = nr_mid_shm_bytes(nmax, 1) - (size_t)nr_mid_tab_bytes();
        gr.warps = (int)std::max<size_t>(1, std::min<size_t>(NR_MID_MAX_WARPS,
                                                             ((size_t)optin - nr_mid_tab_bytes() - 1024) / per_warp));
        gr.smem = nr_mid_shm_bytes(nmax, gr.warps);
        auto it = c->occupancy.find({gr.kfn, gr.smem * 64 + gr.warps});
        int bps;
        if (it == c->occupancy.end()) {
            NR_CUDA_TRY(nr_smem_limit(c->device, gr.kfn, gr.smem));
            NR_CUDA_TRY(cudaOccupancyMaxActiveBlocksPerMultiprocessor(&bps, gr.kfn, 32 * gr.warps, gr.smem));
            c->occupancy[{gr.kfn, gr.smem * 64 + gr.warps}] = bps;
        } else {
            bps = it->second;
        }
        if (bps < 1) return NR_ERR_UNSUPPORTED;
        // a block's two wave buffers; no more blocks than half the free memory holds
        const size_t per_block = 2 * capr * (16 * (size_t)gr.w4 + 8);
        const size_t budget = std::max(per_block, (free_b + c->qbytes) / 2);
        gr.grid = (int)std::max<size_t>(1, std::min<size_t>({(size_t)(j1 - j0), (size_t)bps * c->sms, budget / per_block}));
        slab_need = std::max(slab_need, (size_t)gr.grid * per_block);
        grps.push_back(gr);
        j0 = j1;
    }
    rc = ensure(&c->qbuf, &c->qbytes, slab_need);
    if (rc) return rc;
    NR_CUDA_TRY(cudaEventRecord(c->ev0, s));
    for (const Grp &gr : grps) {
        unsigned char *qb = static_cast<unsigned char *>(c->qbuf);
        NrWarpParams P{};
        P.blob = sb;
        P.inst = reinterpret_cast<const NrSmallGraph *>(sb + off_desc) + gr.j0;
        P.inst_id = reinterpret_cast<const int *>(sb + off_ids) + gr.j0;
        P.n_inst = gr.j1 - gr.j0;
        P.next_inst = reinterpret_cast<int *>(sb);
        P.slab_mask = reinterpret_cast<uint4 *>(qb);
        P.slab_mass = reinterpret_cast<double *>(qb + (size_t)gr.grid * 2 * capr * 16 * gr.w4);
        P.pages = pages;
        P.n_buckets = cfg.n_buckets;
        P.shift = -1;
        P.wave_mode = 1;
        P.eps = cfg.eps;
        P.target = cfg.target;
        P.target_fix = nr_fix_of(cfg.target);
        P.max_nodes = cfg.max_nodes;
        P.out = reinterpret_cast<NrWarpOut *>(sb + off_out);
        P.step_cap = cfg.step_cap;
        P.border = cfg.border;
        P.row_words = gr.row_words;
        NR_CUDA_TRY(cudaMemsetAsync(sb, 0, sizeof(int), s));            // the launch's work counter
        void *args[] = {&P};
        NR_CUDA_TRY(nr_smem_limit(c->device, gr.kfn, gr.smem));
        NR_CUDA_TRY(cudaLaunchKernel(gr.kfn, dim3(gr.grid), dim3(32 * gr.warps), args, gr.smem, s));
    }
    NR_CUDA_TRY(cudaEventRecord(c->ev1, s));
    std::vector<NrWarpOut> hout(k);
    NR_CUDA_TRY(cudaMemcpyAsync(hout.data(), sb + off_out, sizeof(NrWarpOut) * k, cudaMemcpyDeviceToHost, s));
    NR_CUDA_TRY(cudaStreamSynchronize(s));
    float ms = 0.f;
    NR_CUDA_TRY(cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    for (const Grp &gr : grps)
        for (int j = gr.j0; j < gr.j1; ++j) {
            const int i = idx[order[j]];
            if (hout[j].status == NR_LANE_STATUS_CHECK) {
                snprintf(g_internal, sizeof(g_internal), "block kernel check %llu failed on instance %d",
                         (unsigned long long)hout[j].max_wave, i);
                return NR_ERR_INTERNAL;
            }
            nr_result *r = &res[i];
            memset(r, 0, sizeof(*r));
            r->n_nodes = gs[i].n_nodes; r->n_edges = gs[i].n_edges; r->src = srcs[i]; r->dst = dsts[i];
            r->mask_words = std::max(1, (2 * gs[i].n_edges + 31) / 32);
            fill_from_warp(hout[j], cfg, hd[j].w4, r);
            r->kernel = NR_KERNEL_BLOCK;
            r->capacity = capr;
            r->ms = ms;
            r->grid_blocks = gr.grid;
            r->block_threads = 32 * gr.warps;
            r->h2d_bytes = hd[j].blob_bytes + sizeof(NrSmallGraph) + sizeof(int);
            r->d2h_bytes = sizeof(NrWarpOut);
        }
    return NR_OK;
}

// A batch with graphs above 32 nodes, start to end: graphs of up to 32 nodes run
// together on the warp engine, larger ones one at a time on the whole-GPU engine.
static int run_mixed_batch(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                           uint64_t capacity, const nr_options &o, nr_result *res)
{
    std::vector<int> small_idx, wide_idx, handover;
    for (int i = 0; i < n; ++i) (gs[i].n_nodes > NR_SMALL_MAX_N ? wide_idx : small_idx).push_back(i);
    int rc;
    if (!small_idx.empty()) {
        const int m = (int)small_idx.size();
        std::vector<nr_graph> sg(m);
        std::vector<int32_t> ss(m), sd(m);
        std::vector<nr_result> sr(m);
        for (int k = 0; k < m; ++k) {
            sg[k] = gs[small_idx[k]]; ss[k] = srcs[small_idx[k]]; sd[k] = dsts[small_idx[k]];
        }
        std::vector<int> hk;
        rc = run_warp_batch(c, m, sg.data(), ss.data(), sd.data(), batch_cfg(o, capacity), sr.data(), &hk);
        if (rc) return rc;
        for (int k = 0; k < m; ++k) res[small_idx[k]] = sr[k];
        for (int k : hk) handover.push_back(small_idx[k]);
    }
    rc = run_handover(c, handover, gs, srcs, dsts, capacity, o, res);
    if (rc) return rc;
    const uint64_t wcap = std::max<uint64_t>(capacity, 1u << 22);
    // graphs of 33..64 nodes: the 64-bit-row block kernel, one block each, when the run is the lane
    // kernels' kind (breadth-first waves, path branching, plain order) and there are at least a
    // quarter as many of them as SMs (fewer leave most of the GPU to a few blocks: the whole-GPU
    // engine then)
    const WarpRunCfg bcfg = batch_cfg(o, capacity);
    if (bcfg.lane && bcfg.lane2 && !bcfg.fork && !bcfg.learned && bcfg.border != NR_BORDER_LEARNED) {
        std::vector<int> mid_idx, rest;
        for (int i : wide_idx) (mid_ok(gs[i]) ? mid_idx : rest).push_back(i);
        if ((int)mid_idx.size() >= std::max(2, c->sms / 4)) {
            // wave buffers of 2^20 records a block at least (48-80 MB a block; the wide engine's
            // 2^22 a graph would be 200-330 MB for each of up to 152 blocks)
            rc = run_block64(c, mid_idx, gs, srcs, dsts, std::max<uint64_t>(capacity, 1u << 20), bcfg, res);
            if (rc) return rc;
            wide_idx.swap(rest);
        }
    }
    for (int i : wide_idx) {
        nr_result *r = &res[i];
        memset(r, 0, sizeof(*r));
        r->n_nodes = gs[i].n_nodes; r->n_edges = gs[i].n_edges; r->src = srcs[i]; r->dst = dsts[i];
        r->mask_words = std::max(1, (2 * gs[i].n_edges + 31) / 32);
    }
    if (wide_idx.empty()) return NR_OK;
    // breadth-first waves with path branching (run_wide's whole-GPU wave engine): the graphs run
    // side by side, each on its own group of blocks; else one at a time
    const bool buckets = o.bucket_shift >= 0 &&
                         (o.order == NR_ORDER_MAXMASS || (o.order == NR_ORDER_AUTO && o.target_width > 0));
    if (wide_idx.size() > 1 && !buckets && o.order != NR_ORDER_LEARNED && o.branching == NR_BRANCH_PATH)
        return run_grid_wide_multi(c, wide_idx, gs, srcs, dsts, wcap, &o, res);
    for (int i : wide_idx) {
        rc = run_wide(c, &gs[i], srcs[i], dsts[i], wcap, &o, &res[i]);
        if (rc) return rc;
    }
    return NR_OK;
}

// Finish the batch queued on a slot: results, then handed-over instances.
static int slot_finish(nr_context *c, NrSlot &sl)
{
    PhaseClock pc;
    std::vector<int> handover;
    sl.pending = false;
    int rc = warp_finish(c, sl, 0, &handover, pc);
    if (!rc) rc = run_handover(c, handover, sl.gs, sl.srcs, sl.dsts, sl.capacity, sl.opt, sl.res,
                               sl.matrix ? sl.pmat : nullptr);
    return rc;
}

// Finish every batch still in flight (before work that uses slot 0 or swaps the model);
// their statuses wait for their tickets.
void drain(nr_context *c)
{
    for (NrSlot &sl : c->slot)
        if (sl.pending) c->done_rc[sl.ticket] = slot_finish(c, sl);
}

static void record_done(nr_context *c, int64_t ticket, int rc)
{
    c->done_rc[ticket] = rc;
    while (c->done_rc.size() > 64) c->done_rc.erase(c->done_rc.begin());    // waits never made
}

extern "C" int nr_batch_submit(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                               uint64_t capacity, const nr_options *opt, nr_result *res, void *after_stream,
                               int64_t *ticket)
{
    if (!c || !ticket || n < 0 || (n > 0 && (!gs || !srcs || !dsts || !res))) return NR_ERR_INVALID;
    nr_options o;
    if (opt) o = *opt; else nr_options_default(&o);
    std::lock_guard<std::mutex> lock(c->mu);
    const int64_t t = c->next_ticket++;
    *ticket = t;
    if (n == 0) { record_done(c, t, NR_OK); return NR_OK; }
    PhaseClock pc;
    // graphs of up to 32 nodes only (the usual batch): the warp engine's first host pass
    // validates them as it sizes their tables; else the whole batch is validated here first
    bool any_wide = false, uniform = true;   // uniform: one topology (the same CSR arrays) throughout
    for (int i = 0; i < n && !any_wide; ++i) {
        any_wide = gs[i].n_nodes > NR_SMALL_MAX_N;
        uniform = uniform && same_structure_arrays(&gs[i], &gs[0]);
    }
    int n_wide = 0;
    int rc = any_wide ? batch_validate(c, n, gs, srcs, dsts, o, &n_wide) : batch_options_ok(c, o);
    if (rc) { record_done(c, t, rc); return rc; }
    pc.mark("validate");
    NR_CUDA_TRY(cudaSetDevice(c->device));
    if (n_wide) {                             // larger graphs: the whole batch now
        drain(c);
        rc = run_mixed_batch(c, n, gs, srcs, dsts, capacity, o, res);
        record_done(c, t, rc);
        return rc;
    }
    NrSlot &sl = c->slot[(t - 1) % NR_SLOTS];
    if (sl.pending) record_done(c, sl.ticket, slot_finish(c, sl));
    rc = warp_submit(c, sl, 0, n, gs, srcs, dsts, batch_cfg(o, capacity), res, pc,
                     static_cast<cudaStream_t>(after_stream), uniform);
    if (rc) {
        cudaStreamSynchronize(sl.stream);
        record_done(c, t, rc);
        return rc;
    }
    sl.ticket = t;
    sl.pending = true;
    sl.capacity = capacity;
    sl.opt = o;
    return NR_OK;
}

extern "C" int nr_batch_wait(nr_context *c, int64_t ticket)
{
    if (!c) return NR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(c->mu);
    for (NrSlot &sl : c->slot)
        if (sl.pending && sl.ticket == ticket) {
            NR_CUDA_TRY(cudaSetDevice(c->device));
            return slot_finish(c, sl);
        }
    auto it = c->done_rc.find(ticket);
    if (it == c->done_rc.end()) return NR_ERR_INVALID;
    const int rc = it->second;
    c->done_rc.erase(it);
    return rc;
}

// One topology, a matrix of probability sets (nr.h): the topology is checked once, the
// terminals per instance, the matrix for NaN on the device; no per-instance host tables.
extern "C" int nr_batch_submit_matrix(nr_context *c, const nr_graph *topo, int n, const double *p_matrix,
                                      const int32_t *srcs, const int32_t *dsts, uint64_t capacity,
                                      const nr_options *opt, nr_result *res, void *after_stream, int64_t *ticket)
{
    if (!c || !ticket || !topo || n < 0 || (n > 0 && (!p_matrix || !srcs || !dsts || !res))) return NR_ERR_INVALID;
    nr_options o;
    if (opt) o = *opt; else nr_options_default(&o);
    std::lock_guard<std::mutex> lock(c->mu);
    const int64_t t = c->next_ticket++;
    *ticket = t;
    if (n == 0) { record_done(c, t, NR_OK); return NR_OK; }
    int rc = validate_shape(topo, srcs[0], dsts[0]);
    if (!rc) rc = validate_structure(topo);
    if (!rc && topo->n_nodes > NR_SMALL_MAX_N) rc = NR_ERR_UNSUPPORTED;
    if (!rc) rc = batch_options_ok(c, o);
    if (rc) { record_done(c, t, rc); return rc; }
    NR_CUDA_TRY(cudaSetDevice(c->device));
    PhaseClock pc;
    NrSlot &sl = c->slot[(t - 1) % NR_SLOTS];
    if (sl.pending) record_done(c, sl.ticket, slot_finish(c, sl));
    rc = warp_submit(c, sl, 0, n, topo, srcs, dsts, batch_cfg(o, capacity), res, pc,
                     static_cast<cudaStream_t>(after_stream), true, p_matrix);
    if (rc) {
        cudaStreamSynchronize(sl.stream);
        sl.matrix = false;
        record_done(c, t, rc);
        return rc;
    }
    sl.ticket = t;
    sl.pending = true;
    sl.capacity = capacity;
    sl.opt = o;
    return NR_OK;
}

extern "C" int nr_reliability_batch_matrix(nr_context *c, const nr_graph *topo, int n, const double *p_matrix,
                                           const int32_t *srcs, const int32_t *dsts, uint64_t capacity,
                                           const nr_options *opt, nr_result *res)
{
    int64_t t = 0;
    const int rc = nr_batch_submit_matrix(c, topo, n, p_matrix, srcs, dsts, capacity, opt, res, nullptr, &t);
    if (rc) return rc;
    return nr_batch_wait(c, t);
}

extern "C" int nr_reliability_batch(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs,
                                    const int32_t *dsts, uint64_t capacity, const nr_options *opt,
                                    nr_result *res)
{
    if (!c || n < 0 || (n > 0 && (!gs || !srcs || !dsts || !res))) return NR_ERR_INVALID;
    int64_t t = 0;
    const int rc = nr_batch_submit(c, n, gs, srcs, dsts, capacity, opt, res, nullptr, &t);
    const int rw = nr_batch_wait(c, t);
    return rc ? rc : rw;
}

// Autotuner: time candidate warp-engine settings on (a sample of) the batch
// and return the fastest.  Candidates: bucket resolution (2^shift buckets per
// octave, shift 0..2, or one bucket = breadth-first waves; the "bucket count"), pages per warp (the pop chunk:
// how much of a bucket a warp holds and takes at a time), and warps per
// block.  Every candidate gives a valid result (exact counts for exhaustive
// runs; for truncated runs a bracket whose width meets the target); the
// choice only changes time, and for truncated runs where the stop falls.
extern "C" int nr_autotune(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs, const int32_t *dsts,
                           uint64_t capacity, const nr_options *opt, nr_options *best, double *best_ms)
{
    if (!c || n <= 0 || !gs || !srcs || !dsts || !best) return NR_ERR_INVALID;
    nr_options base;
    if (opt) base = *opt; else nr_options_default(&base);
    const int sample = std::min(n, 4096);
    std::vector<nr_result> res(sample);
    const bool exhaustive = !(base.target_width > 0) && base.order != NR_ORDER_MAXMASS &&
                            base.order != NR_ORDER_LEARNED;
    // The bucket resolution is searched only when the caller leaves the order to the engine:
    // NR_ORDER_WAVES holds one bucket (breadth-first waves), NR_ORDER_MAXMASS the caller's shift.
    const int shifts_t[] = {-1, 0, 1, 2};   // -1: one bucket, i.e. breadth-first waves
    const int shifts_e[] = {base.order == NR_ORDER_WAVES ? -1 : base.bucket_shift};
    const bool held = exhaustive || base.order == NR_ORDER_WAVES || base.order == NR_ORDER_MAXMASS ||
                      base.order == NR_ORDER_LEARNED;
    const int *shifts = held ? shifts_e : shifts_t;
    const int n_shift = held ? 1 : 4;
    // pages per warp: 64 and 512 (small and medium queues), 4096 for instances whose waves
    // outgrow 512 pages; with a capacity, candidates above it collapse onto it
    const uint64_t pages_c[] = {64, 512, 4096};
    const int wpb_c[] = {2, 4, 8};
    // A candidate is ranked by the instances whose queue spilled (a spill widens the bracket, so
    // fewer is better whatever the time), then by device time: the best of three runs, and for
    // the three leaders three more after every candidate has run once (clock and cache state
    // drift over a search).
    struct Cand { nr_options o; uint64_t cap; int spills; double t; };
    std::vector<Cand> cands;
    auto time_it = [&](Cand &k, int reps) -> int {
        for (int rep = 0; rep < reps; ++rep) {
            int rc = nr_reliability_batch(c, sample, gs, srcs, dsts, k.cap, &k.o, res.data());
            if (rc) return rc;
            double ms = 0;
            bool warp_only = true;
            int spills = 0;
            for (int i = 0; i < sample; ++i) {
                if (res[i].engine != NR_ENGINE_WARP) warp_only = false;
                spills += res[i].spilled != 0;
                ms = std::max(ms, res[i].ms);
            }
            if (!warp_only) ms = 1e300;      // a hand-over costs a full extra solve
            k.t = std::min(k.t, ms);
            k.spills = spills;
        }
        return NR_OK;
    };
    for (int si = 0; si < n_shift; ++si)
        for (int pi = 0; pi < 3; ++pi)
            for (int wpb : wpb_c) {
                const uint64_t pg = pages_c[pi];
                if (pi > 0 && capacity && capacity <= pages_c[pi - 1] * NR_PAGE) continue;
                Cand k;
                k.o = base;
                k.o.bucket_shift = shifts[si];
                k.o.n_buckets = held && base.n_buckets > 0 ? base.n_buckets : 64 << std::max(0, shifts[si]);
                k.o.warps_per_block = wpb;
                k.o.max_nodes = base.max_nodes;
                // the queue size timed: pages_per_warp applies to calls with capacity 0
                k.o.pages_per_warp = (int32_t)std::min<uint64_t>(pg, capacity ? (capacity + NR_PAGE - 1) / NR_PAGE : pg);
                k.cap = capacity ? std::min<uint64_t>(capacity, pg * NR_PAGE) : pg * NR_PAGE;
                k.spills = 0;
                k.t = 1e300;
                const int rc = time_it(k, 3);
                if (rc) return rc;
                cands.push_back(k);
            }
    auto better = [](const Cand &a, const Cand &b) { return a.spills != b.spills ? a.spills < b.spills : a.t < b.t; };
    std::sort(cands.begin(), cands.end(), better);
    for (size_t i = 0; i < std::min<size_t>(3, cands.size()); ++i) {
        const int rc = time_it(cands[i], 3);
        if (rc) return rc;
    }
    std::sort(cands.begin(), cands.begin() + std::min<size_t>(3, cands.size()), better);
    *best = cands[0].o;
    if (best_ms) *best_ms = cands[0].t;
    return NR_OK;
}

// Install the learned scorer's parameters (flat FP32, nr_mlp_param_count()
// floats) on the context; NR_ORDER_LEARNED calls use its BF16 copy.
extern "C" int nr_context_set_model(nr_context *c, const float *params)
{
    if (!c || !params) return NR_ERR_INVALID;
    std::lock_guard<std::mutex> lock(c->mu);
    drain(c);                          // finish batches in flight: slot 0 and the model are used here
    NR_CUDA_TRY(cudaSetDevice(c->device));
    int rc = nr_mlp_upload(params, &c->model, &c->mlp, c->stream);
    if (rc) return rc;
    NR_CUDA_TRY(cudaStreamSynchronize(c->stream));
    c->has_model = true;
    return NR_OK;
}

// Solve a batch with the warp engine (options as nr_reliability_batch) and
// record every child it queues: features (16 floats), mask words (stride 32),
// mass and instance index, up to max_items.  *count receives how many were
// recorded (children past max_items are not recorded).  Training data for the
// learned scorer.
extern "C" int nr_collect_children(nr_context *c, int n, const nr_graph *gs, const int32_t *srcs,
                                   const int32_t *dsts, uint64_t capacity, const nr_options *opt,
                                   uint64_t max_items, float *feat, uint32_t *masks, double *mass, int32_t *inst,
                                   uint64_t *count, nr_result *res)
{
    if (!c || n <= 0 || !gs || !srcs || !dsts || !feat || !masks || !mass || !inst || !count || !res)
        return NR_ERR_INVALID;
    nr_options o;
    if (opt) o = *opt; else nr_options_default(&o);
    for (int i = 0; i < n; ++i) {
        memset(&res[i], 0, sizeof(nr_result));
        int rc = validate(&gs[i], srcs[i], dsts[i]);
        if (rc) return rc;
        if (gs[i].n_nodes > NR_SMALL_MAX_N) return NR_ERR_UNSUPPORTED;
    }
    std::lock_guard<std::mutex> lock(c->mu);
    drain(c);                          // finish batches in flight: slot 0 and the model are used here
    NR_CUDA_TRY(cudaSetDevice(c->device));
    if (o.order == NR_ORDER_LEARNED && !c->has_model) return NR_ERR_INVALID;
    if (o.branching != NR_BRANCH_PATH) return NR_ERR_UNSUPPORTED;    // features describe path children
    const bool exhaustive = !(o.target_width > 0) && o.order != NR_ORDER_MAXMASS && o.order != NR_ORDER_LEARNED;
    WarpRunCfg cfg = warp_cfg(&o, capacity, exhaustive);
    cfg.escalate = 0;                 // collect from whatever the warp engine reaches
    const int stride = 32;
    unsigned char *buf = nullptr;
    const size_t bytes = max_items * (NR_FEAT * sizeof(float) + stride * sizeof(uint32_t) + sizeof(double) +
                                      sizeof(int)) + 64;
    if (cudaMalloc(&buf, bytes) != cudaSuccess) { cudaGetLastError(); return NR_ERR_NOMEM; }
    WarpDump d;
    d.count = reinterpret_cast<unsigned long long *>(buf);
    d.feat = reinterpret_cast<float *>(buf + 64);
    d.mask = reinterpret_cast<uint32_t *>(d.feat + max_items * NR_FEAT);
    d.mass = reinterpret_cast<double *>(d.mask + max_items * stride);
    d.inst = reinterpret_cast<int *>(d.mass + max_items);
    d.cap = max_items;
    d.stride = stride;
    cfg.dump = &d;
    int rc = NR_OK;
    unsigned long long got = 0;
    // the counter must be zero before the batch's own streams start
    if (cudaMemsetAsync(buf, 0, 64, c->stream) != cudaSuccess || cudaStreamSynchronize(c->stream) != cudaSuccess)
        rc = NR_ERR_CUDA;
    std::vector<int> handover;
    if (!rc) rc = run_warp_batch(c, n, gs, srcs, dsts, cfg, res, &handover);
    if (!rc) {
        cudaStream_t s = c->stream;
        cudaMemcpyAsync(&got, d.count, sizeof(got), cudaMemcpyDeviceToHost, s);
        cudaStreamSynchronize(s);
        const unsigned long long k = std::min<unsigned long long>(got, max_items);
        if (k) {
            cudaMemcpyAsync(feat, d.feat, k * NR_FEAT * sizeof(float), cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(masks, d.mask, k * stride * sizeof(uint32_t), cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(mass, d.mass, k * sizeof(double), cudaMemcpyDeviceToHost, s);
            cudaMemcpyAsync(inst, d.inst, k * sizeof(int), cudaMemcpyDeviceToHost, s);
        }
        if (cudaStreamSynchronize(s) != cudaSuccess) { cudaGetLastError(); rc = NR_ERR_CUDA; }
        *count = k;
    }
    cudaFree(buf);
    return rc;
}

