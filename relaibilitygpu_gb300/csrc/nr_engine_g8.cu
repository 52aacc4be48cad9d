// nr_engine_g8.cu -- kernels for graphs with up to 8 nodes (lane groups of 8).
// One translation unit per group width keeps the build parallel.
#include "nr_grid.cuh"
#include "nr_warp.cuh"

#define NR_W4_CASES(KERNEL)                              \
    switch (w4) {                                        \
    case 1: return (const void *)KERNEL<8, 1>;           \
    case 2: return (const void *)KERNEL<8, 2>;           \
    case 3: return (const void *)KERNEL<8, 3>;           \
    case 4: return (const void *)KERNEL<8, 4>;           \
    case 5: return (const void *)KERNEL<8, 5>;           \
    case 6: return (const void *)KERNEL<8, 6>;           \
    case 7: return (const void *)KERNEL<8, 7>;           \
    case 8: return (const void *)KERNEL<8, 8>;           \
    default: return nullptr;                             \
    }

const void *nr_grid_kernel_ptr_g8(int w4) { NR_W4_CASES(nr_grid_kernel) }
const void *nr_warp_kernel_ptr_g8(int w4) { NR_W4_CASES(nr_warp_kernel) }
