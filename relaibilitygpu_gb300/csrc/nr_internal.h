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

// Exact mass sums: a 192-bit unsigned integer A standing for A / 2^190.
// Adding an FP64 mass places its 53-bit significand exactly (masses down to
// 2^-137 are exact; smaller ones are truncated by less than 2^-190), so sums
// do not depend on the order of the additions and subtraction is exact too.
#define NR_FIX_FRAC 190
struct NrFix {
    unsigned long long w0, w1, w2;
};

// Per-block result partials written at kernel exit (no single-address atomics;
// the host adds them).
struct NrPartial {
    NrFix R;                    // all-up leaf mass
    NrFix et;                   // eps-truncated mass
    NrFix es;                   // spilled mass
    NrFix q;                    // mass still queued when a target width stopped the run
    unsigned long long nodes, leaves, dead, truncated, spilled, pad;
};

// Graph tables of one instance (small engines) in two parts:
//   per instance, at blob_off:   p[E] (double); the root mask is derived from p on the device;
//   per topology, at struct_off: eid_tab[G*G] (u16, arc u->v at u*G+v),
//                                in_start[n+1] (int), in_list[n_in] (u32 = eid << 8 | u).
// Instances with the same topology share one structural part.  When both parts
// are one blob, struct_off == blob_off.  Every section starts 16-byte aligned;
// blob_bytes is the size of the instance's own part(s).
struct NrSmallGraph {
    int n, e, w4, src, dst, n_in;
    int off_p, off_eid, off_start, off_list, blob_bytes;
    int rows;                   // rows carried in queue records: 0 no (rebuilt from the mask),
                                // 1 undirected simple graph, 2 directed simple graph
    int off_root_rows;          // every node's in-neighbour row (all arcs) for the lane kernels'
                                // roots: n <= 16, 16 bits each, two to a word; n <= 32, one a
                                // word (32 words; structural part; 0 when absent)
    long long blob_off;
    long long struct_off;
};

struct NrGridParams {
    NrSmallGraph g;
    const unsigned char *blob;        // graph tables in global memory
    uint4 *mask[2];                   // ping-pong wave buffers: [capacity][w4] 16-byte blocks
    double *mass[2];                  // [capacity]
    uint4 *rows[2];                   // one lane a subproblem: [capacity][2] not-down rows (else nullptr)
    unsigned long long capacity;
    unsigned long long *wave_count;   // [max_waves + 1]; wave_count[0] = 1 (the root)
    int max_waves;
    unsigned *bar_count;
    unsigned *bar_gen;
    int *status;
    NrPartial *partials;              // [gridDim.x]
    double eps;
    long long timeout_ns;
    int fork;                         // 1: fork branching on the most reliable path edge
    int border;                       // NR_BORDER_*: the order a path's UNKNOWN edges are branched in
    int test_fault;                   // 1 (failure-path tests only): block 0 leaves before its
                                      // first grid barrier, so the others' bounded waits run out
};

// host helpers for NrFix (nr_api.cu)
NrFix nr_fix_from_double_host(double m);
double nr_fix_to_double_host(const NrFix &a);
void nr_fix_add_host(NrFix &a, const NrFix &b);

// host-side helpers implemented in nr_engine_*.cu
int nr_launch_grid_small(int G, const NrGridParams &p, int grid, int block, size_t smem,
                         cudaStream_t stream);
int nr_grid_small_occupancy(int G, int w4, int block, size_t smem, int *blocks_per_sm);

// Sets a kernel's dynamic shared-memory limit on a device when it differs from
// the value last set through this function (nr_api.cu).
cudaError_t nr_smem_limit(int device, const void *kfn, size_t bytes);
