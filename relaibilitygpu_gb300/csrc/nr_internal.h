// nr_internal.h -- structures shared by the engine's host code and kernels.
#pragma once

#include <cuda_runtime.h>
#include <stdint.h>

#include "nr.h"

// Small-graph engines: one lane per node, so n_nodes <= 32.
#define NR_SMALL_MAX_N 32
// Mask records are 16-byte blocks; 8 blocks = 32 words = 512 edges.
#define NR_MAX_W4 8
#define NR_BLOCK_THREADS 256

// device status bits (OR-ed into a status word)
#define NR_DEV_ERR_TIMEOUT 1
#define NR_DEV_ERR_BOUNDS 2
#define NR_DEV_ERR_WAVES 4

// Per-block result partials written at kernel exit (no single-address atomics
// on the sums; the host merges them with two-sum in block order).
struct NrPartial {
    double R_hi, R_lo;          // all-up leaf mass
    double et_hi, et_lo;        // eps-truncated mass
    double es_hi, es_lo;        // spilled mass
    unsigned long long nodes, leaves, dead, truncated, spilled, pad;
};

// Graph tables of one instance (small engines), laid out in one blob:
// p[E], q[E] (double), eid_tab[G*G] (u16, arc u->v at u*G+v), in_start[n+1]
// (int), in_list[n_in] (u32 = eid << 8 | u), root mask (4*w4 words).
// Offsets are relative to blob_off; every section starts 16-byte aligned.
struct NrSmallGraph {
    int n, e, w4, src, dst, n_in;
    int off_p, off_q, off_eid, off_start, off_list, off_root, blob_bytes;
    long long blob_off;
};

struct NrGridParams {
    NrSmallGraph g;
    const unsigned char *blob;        // graph tables in global memory
    uint4 *mask[2];                   // ping-pong wave buffers: [capacity][w4] 16-byte blocks
    double *mass[2];                  // [capacity]
    unsigned long long capacity;
    unsigned long long *wave_count;   // [max_waves + 1]; wave_count[0] = 1 (the root)
    int max_waves;
    unsigned *bar_count;
    unsigned *bar_gen;
    int *status;
    NrPartial *partials;              // [gridDim.x]
    double eps;
    long long timeout_ns;
};

// compensated summation, kept free of contraction by the _rn intrinsics
struct NrKs {
    double hi, lo;
};

// host-side helpers implemented in nr_engine_*.cu
int nr_launch_grid_small(int G, const NrGridParams &p, int grid, int block, size_t smem,
                         cudaStream_t stream);
int nr_grid_small_occupancy(int G, int w4, int block, size_t smem, int *blocks_per_sm);
