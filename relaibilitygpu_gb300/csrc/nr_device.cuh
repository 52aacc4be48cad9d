// nr_device.cuh -- device helpers shared by the engine kernels.
#pragma once

#include <string.h>

#include "nr_internal.h"

#define NR_FULL 0xffffffffu

__host__ __device__ __forceinline__ NrFix nr_fix_zero()
{
    NrFix r;
    r.w0 = r.w1 = r.w2 = 0ull;
    return r;
}

// exact value of a non-negative finite double, as a 192-bit fixed-point number
__host__ __device__ __forceinline__ NrFix nr_fix_of(double m)
{
    unsigned long long bits;
#ifdef __CUDA_ARCH__
    bits = (unsigned long long)__double_as_longlong(m);
#else
    memcpy(&bits, &m, 8);
#endif
    NrFix r = nr_fix_zero();
    const int ex = (int)((bits >> 52) & 0x7ff);
    unsigned long long M = bits & 0xfffffffffffffull;
    int e;
    if (ex == 0) {
        e = -1074;
    } else {
        M |= 1ull << 52;
        e = ex - 1075;
    }
    if (M == 0ull) return r;
    const int s = e + NR_FIX_FRAC;
    if (s >= 0) {
        const int k = s >> 6, b = s & 63;
        const unsigned long long lo = M << b;
        const unsigned long long hi = b ? (M >> (64 - b)) : 0ull;
        if (k == 0) { r.w0 = lo; r.w1 = hi; }
        else if (k == 1) { r.w1 = lo; r.w2 = hi; }
        else if (k == 2) { r.w2 = lo; }
    } else if (-s < 64) {
        r.w0 = M >> (-s);
    }
    return r;
}

__host__ __device__ __forceinline__ void nr_fix_add(NrFix &a, const NrFix &b)
{
#ifdef __CUDA_ARCH__
    // one carry chain through the three words
    asm("add.cc.u64 %0, %0, %3;\n\t"
        "addc.cc.u64 %1, %1, %4;\n\t"
        "addc.u64 %2, %2, %5;"
        : "+l"(a.w0), "+l"(a.w1), "+l"(a.w2)
        : "l"(b.w0), "l"(b.w1), "l"(b.w2));
#else
    const unsigned long long w0 = a.w0 + b.w0;
    const unsigned long long c0 = w0 < a.w0;
    const unsigned long long t1 = a.w1 + b.w1;
    unsigned long long c1 = t1 < a.w1;
    const unsigned long long w1 = t1 + c0;
    c1 += w1 < t1;
    a.w2 = a.w2 + b.w2 + c1;
    a.w1 = w1;
    a.w0 = w0;
#endif
}

__host__ __device__ __forceinline__ void nr_fix_sub(NrFix &a, const NrFix &b)
{
#ifdef __CUDA_ARCH__
    asm("sub.cc.u64 %0, %0, %3;\n\t"
        "subc.cc.u64 %1, %1, %4;\n\t"
        "subc.u64 %2, %2, %5;"
        : "+l"(a.w0), "+l"(a.w1), "+l"(a.w2)
        : "l"(b.w0), "l"(b.w1), "l"(b.w2));
#else
    const unsigned long long w0 = a.w0 - b.w0;
    const unsigned long long b0 = a.w0 < b.w0;
    const unsigned long long t1 = a.w1 - b.w1;
    unsigned long long b1 = a.w1 < b.w1;
    const unsigned long long w1 = t1 - b0;
    b1 += t1 < b0;
    a.w2 = a.w2 - b.w2 - b1;
    a.w1 = w1;
    a.w0 = w0;
#endif
}

__host__ __device__ __forceinline__ bool nr_fix_le(const NrFix &a, const NrFix &b)
{
    if (a.w2 != b.w2) return a.w2 < b.w2;
    if (a.w1 != b.w1) return a.w1 < b.w1;
    return a.w0 <= b.w0;
}

__device__ __forceinline__ void nr_fix_add_mass(NrFix &a, double m) { nr_fix_add(a, nr_fix_of(m)); }

__device__ __forceinline__ NrFix nr_fix_shfl_xor(const NrFix &a, int off)
{
    NrFix o;
    o.w0 = __shfl_xor_sync(NR_FULL, a.w0, off);
    o.w1 = __shfl_xor_sync(NR_FULL, a.w1, off);
    o.w2 = __shfl_xor_sync(NR_FULL, a.w2, off);
    return o;
}

// exact warp total, returned on every lane
__device__ __forceinline__ NrFix nr_fix_warp_sum(NrFix a)
{
    for (int off = 16; off > 0; off >>= 1) {
        const NrFix o = nr_fix_shfl_xor(a, off);
        nr_fix_add(a, o);
    }
    return a;
}

// exact warp total of a sum that is mostly zero: one vote when every lane holds zero
__device__ __forceinline__ NrFix nr_fix_warp_sum_sparse(const NrFix &a)
{
    if (!__any_sync(NR_FULL, (a.w0 | a.w1 | a.w2) != 0ull)) return nr_fix_zero();
    return nr_fix_warp_sum(a);
}

// warp total of a 64-bit count (modulo 2^64) by three integer reductions of 21/21/22-bit limbs
// (each limb's total stays below 2^27)
__device__ __forceinline__ unsigned long long nr_warp_sum_u64r(unsigned long long x)
{
    const unsigned a = __reduce_add_sync(NR_FULL, (unsigned)(x & 0x1fffffull));
    const unsigned b = __reduce_add_sync(NR_FULL, (unsigned)((x >> 21) & 0x1fffffull));
    const unsigned c = __reduce_add_sync(NR_FULL, (unsigned)(x >> 42));
    return (unsigned long long)a + ((unsigned long long)b << 21) + ((unsigned long long)c << 42);
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
// nblocks: the blocks that meet at this barrier (all of the grid, or one instance's group of
// blocks in a launch that runs several instances).
__device__ __forceinline__ bool nr_grid_sync(unsigned *count, unsigned *gen, int *status,
                                             long long timeout_ns, unsigned nblocks = 0)
{
    if (nblocks == 0) nblocks = gridDim.x;
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
        if (prev == nblocks - 1) {
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
__device__ __forceinline__ void nr_block_partial(NrPartial *out, NrFix R, NrFix et, NrFix es, NrFix q,
                                                 unsigned long long nodes, unsigned long long leaves,
                                                 unsigned long long dead, unsigned long long trunc,
                                                 unsigned long long spilled)
{
    __shared__ NrFix s_fx[NR_BLOCK_THREADS / 32][4];
    __shared__ unsigned long long s_c[NR_BLOCK_THREADS / 32][5];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    R = nr_fix_warp_sum(R);
    et = nr_fix_warp_sum(et);
    es = nr_fix_warp_sum(es);
    q = nr_fix_warp_sum(q);
    for (int off = 16; off > 0; off >>= 1) {
        nodes += __shfl_xor_sync(NR_FULL, nodes, off);
        leaves += __shfl_xor_sync(NR_FULL, leaves, off);
        dead += __shfl_xor_sync(NR_FULL, dead, off);
        trunc += __shfl_xor_sync(NR_FULL, trunc, off);
        spilled += __shfl_xor_sync(NR_FULL, spilled, off);
    }
    if (lane == 0) {
        s_fx[warp][0] = R; s_fx[warp][1] = et; s_fx[warp][2] = es; s_fx[warp][3] = q;
        s_c[warp][0] = nodes; s_c[warp][1] = leaves; s_c[warp][2] = dead;
        s_c[warp][3] = trunc; s_c[warp][4] = spilled;
    }
    __syncthreads();
    if (threadIdx.x == 0) {
        NrFix r = nr_fix_zero(), a = nr_fix_zero(), b = nr_fix_zero(), qq = nr_fix_zero();
        unsigned long long c[5] = {0, 0, 0, 0, 0};
        for (int w = 0; w < (int)(blockDim.x >> 5); ++w) {
            nr_fix_add(r, s_fx[w][0]);
            nr_fix_add(a, s_fx[w][1]);
            nr_fix_add(b, s_fx[w][2]);
            nr_fix_add(qq, s_fx[w][3]);
            for (int k = 0; k < 5; ++k) c[k] += s_c[w][k];
        }
        out->R = r; out->et = a; out->es = b; out->q = qq;
        out->nodes = c[0]; out->leaves = c[1]; out->dead = c[2];
        out->truncated = c[3]; out->spilled = c[4]; out->pad = 0;
    }
}

// Sum of one NrFix per thread over the block, returned on every thread (exact,
// so every block that sums the same values gets the same bits).
__device__ __forceinline__ NrFix nr_block_fix_sum(NrFix v)
{
    __shared__ NrFix s_w[32];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5, nw = (int)(blockDim.x >> 5);
    v = nr_fix_warp_sum(v);
    __syncthreads();                       // s_w may still be read by an earlier call
    if (lane == 0) s_w[warp] = v;
    __syncthreads();
    NrFix t = nr_fix_zero();
    for (int w = 0; w < nw; ++w) nr_fix_add(t, s_w[w]);
    return t;
}

// Bucket of a mass: 2^shift buckets per factor of two, highest masses first;
// the last bucket takes every smaller mass.  Shift < 0 or one bucket: 0.
__device__ __forceinline__ int nr_bucket(double m, int shift, int nb)
{
    if (shift < 0 || nb <= 1) return 0;
    const unsigned long long bits = (unsigned long long)__double_as_longlong(m);
    const long long key = (long long)(bits >> (52 - shift));
    long long b = (1023LL << shift) - key;
    b = b < 0 ? 0 : b;
    b = b > nb - 1 ? nb - 1 : b;
    return (int)b;
}

// Stage the graph tables into shared memory (16-byte copies; blob_bytes is a multiple of 16).
__device__ __forceinline__ void nr_stage_blob(unsigned char *dst, const unsigned char *src, int bytes)
{
    const uint4 *s = reinterpret_cast<const uint4 *>(src);
    uint4 *d = reinterpret_cast<uint4 *>(dst);
    for (int i = threadIdx.x; i < bytes / 16; i += blockDim.x) d[i] = __ldg(s + i);
}
