// nr_engine_g16.cu -- kernels for graphs with up to 16 nodes (lane groups of 16).
// One translation unit per group width keeps the build parallel.
#include "nr_grid.cuh"

const void *nr_grid_kernel_ptr_g16(int w4)
{
    switch (w4) {
    case 1: return (const void *)nr_grid_kernel<16, 1>;
    case 2: return (const void *)nr_grid_kernel<16, 2>;
    case 3: return (const void *)nr_grid_kernel<16, 3>;
    case 4: return (const void *)nr_grid_kernel<16, 4>;
    case 5: return (const void *)nr_grid_kernel<16, 5>;
    case 6: return (const void *)nr_grid_kernel<16, 6>;
    case 7: return (const void *)nr_grid_kernel<16, 7>;
    case 8: return (const void *)nr_grid_kernel<16, 8>;
    default: return nullptr;
    }
}
