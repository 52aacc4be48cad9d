// nr_engine_g8.cu -- kernels for graphs with up to 8 nodes (lane groups of 8).
// One translation unit per group width keeps the build parallel.
#include "nr_grid.cuh"
#include "nr_warp.cuh"

#define NR_W4_CASES(KERNEL, ...)                         \
    switch (w4) {                                        \
    case 1: return (const void *)KERNEL<8, 1 __VA_ARGS__>;   \
    case 2: return (const void *)KERNEL<8, 2 __VA_ARGS__>;   \
    case 3: return (const void *)KERNEL<8, 3 __VA_ARGS__>;   \
    case 4: return (const void *)KERNEL<8, 4 __VA_ARGS__>;   \
    case 5: return (const void *)KERNEL<8, 5 __VA_ARGS__>;   \
    case 6: return (const void *)KERNEL<8, 6 __VA_ARGS__>;   \
    case 7: return (const void *)KERNEL<8, 7 __VA_ARGS__>;   \
    case 8: return (const void *)KERNEL<8, 8 __VA_ARGS__>;   \
    default: return nullptr;                             \
    }

const void *nr_grid_kernel_ptr_g8(int w4) { NR_W4_CASES(nr_grid_kernel) }
const void *nr_grid_fork_kernel_ptr_g8(int w4) { NR_W4_CASES(nr_grid_kernel, , true) }
const void *nr_warp_kernel_ptr_g8(int w4) { NR_W4_CASES(nr_warp_kernel) }
const void *nr_warp_learn_kernel_ptr_g8(int w4) { NR_W4_CASES(nr_warp_kernel, , true) }
const void *nr_warp_fork_kernel_ptr_g8(int w4) { NR_W4_CASES(nr_warp_kernel, , false, true) }
