// nr_device.cuh -- device helpers shared by the engine kernels.
#pragma once

#include "nr_internal.h"

#define NR_FULL 0xffffffffu

__device__ __forceinline__ void nr_ks_add(NrKs &s, double x)
{
    double t = __dadd_rn(s.hi, x);
    double bp = __dadd_rn(t, -s.hi);
    double err = __dadd_rn(__dadd_rn(s.hi, -__dadd_rn(t, -bp)), __dadd_rn(x, -bp));
    s.hi = t;
    s.lo = __dadd_rn(s.lo, err);
}

__device__ __forceinline__ void nr_ks_merge(NrKs &s, const NrKs &o)
{
    nr_ks_add(s, o.hi);
    nr_ks_add(s, o.lo);
}

__device__ __forceinline__ NrKs nr_ks_shfl_down(const NrKs &s, int off)
{
    NrKs o;
    o.hi = __shfl_down_sync(NR_FULL, s.hi, off);
    o.lo = __shfl_down_sync(NR_FULL, s.lo, off);
    return o;
}

__device__ __forceinline__ long long nr_globaltimer()
{
    long long t;
    asm volatile("mov.u64 %0, %%globaltimer;" : "=l"(t));
    return t;
}

// Grid-wide barrier for a cooperative launch. Every wait is bounded: a block
// that sees no other block arrive for timeout_ns (or sees another block's
// error) gives up, sets NR_DEV_ERR_TIMEOUT and returns false, and the caller
// leaves its loop so the kernel still ends.
__device__ __forceinline__ bool nr_grid_sync(unsigned *count, unsigned *gen, int *status,
                                             long long timeout_ns)
{
    __shared__ int s_ok;
    __syncthreads();
    if (threadIdx.x == 0) {
        volatile unsigned *vgen = gen;
        volatile unsigned *vcount = count;
        volatile int *vstatus = status;
        unsigned g0 = *vgen;
        __threadfence();
        unsigned prev = atomicAdd(count, 1u);
        int ok = 1;
        if (prev == gridDim.x - 1) {
            *vcount = 0;
            __threadfence();
            atomicAdd(gen, 1u);
        } else {
            long long t0 = nr_globaltimer();
            unsigned last = prev + 1;
            while (*vgen == g0) {
                __nanosleep(100);
                unsigned c = *vcount;
                long long t = nr_globaltimer();
                if (c != last) { last = c; t0 = t; }
                if (*vstatus != 0) { ok = 0; break; }
                if (t - t0 > timeout_ns) {
                    atomicOr(status, NR_DEV_ERR_TIMEOUT);
                    ok = 0;
                    break;
                }
            }
        }
        __threadfence();
        s_ok = ok;
    }
    __syncthreads();
    return s_ok != 0;
}

// Block reduction of the per-lane sums and counters into one NrPartial.
__device__ __forceinline__ void nr_block_partial(NrPartial *out, NrKs R, NrKs et, NrKs es,
                                                 unsigned long long nodes, unsigned long long leaves,
                                                 unsigned long long dead, unsigned long long trunc,
                                                 unsigned long long spilled)
{
    __shared__ NrKs s_ks[NR_BLOCK_THREADS / 32][3];
    __shared__ unsigned long long s_c[NR_BLOCK_THREADS / 32][5];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int off = 16; off > 0; off >>= 1) {
        NrKs a = nr_ks_shfl_down(R, off), b = nr_ks_shfl_down(et, off), c = nr_ks_shfl_down(es, off);
        nr_ks_merge(R, a);
        nr_ks_merge(et, b);
        nr_ks_merge(es, c);
        nodes += __shfl_down_sync(NR_FULL, nodes, off);
        leaves += __shfl_down_sync(NR_FULL, leaves, off);
        dead += __shfl_down_sync(NR_FULL, dead, off);
        trunc += __shfl_down_sync(NR_FULL, trunc, off);
        spilled += __shfl_down_sync(NR_FULL, spilled, off);
    }
    if (lane == 0) {
        s_ks[warp][0] = R; s_ks[warp][1] = et; s_ks[warp][2] = es;
        s_c[warp][0] = nodes; s_c[warp][1] = leaves; s_c[warp][2] = dead;
        s_c[warp][3] = trunc; s_c[warp][4] = spilled;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        NrKs r = {0, 0}, a = {0, 0}, b = {0, 0};
        unsigned long long c[5] = {0, 0, 0, 0, 0};
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            nr_ks_merge(r, s_ks[w][0]);
            nr_ks_merge(a, s_ks[w][1]);
            nr_ks_merge(b, s_ks[w][2]);
            for (int k = 0; k < 5; ++k) c[k] += s_c[w][k];
        }
        out->R_hi = r.hi; out->R_lo = r.lo;
        out->et_hi = a.hi; out->et_lo = a.lo;
        out->es_hi = b.hi; out->es_lo = b.lo;
        out->nodes = c[0]; out->leaves = c[1]; out->dead = c[2];
        out->truncated = c[3]; out->spilled = c[4]; out->pad = 0;
    }
}

// Stage the graph tables into shared memory (16-byte copies; blob_bytes is a multiple of 16).
__device__ __forceinline__ void nr_stage_blob(unsigned char *dst, const unsigned char *src, int bytes)
{
    const uint4 *s = reinterpret_cast<const uint4 *>(src);
    uint4 *d = reinterpret_cast<uint4 *>(dst);
    for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) d[i] = __ldg(s + i);
}
