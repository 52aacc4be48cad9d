// nr_engine_wide_multi.cu -- the whole-GPU wave kernel that runs several graphs above 32 nodes
// side by side (a batch's large graphs), one per mask width; its own translation unit keeps the
// build parallel.
#include "nr_wide.cuh"

const void *nr_grid_wide_multi_kernel_ptr(int w4)
{
    switch (w4) {
    case 1: return (const void *)nr_grid_wide_multi_kernel<1>;
    case 2: return (const void *)nr_grid_wide_multi_kernel<2>;
    case 3: return (const void *)nr_grid_wide_multi_kernel<3>;
    case 4: return (const void *)nr_grid_wide_multi_kernel<4>;
    case 5: return (const void *)nr_grid_wide_multi_kernel<5>;
    case 6: return (const void *)nr_grid_wide_multi_kernel<6>;
    case 7: return (const void *)nr_grid_wide_multi_kernel<7>;
    case 8: return (const void *)nr_grid_wide_multi_kernel<8>;
    case 9: return (const void *)nr_grid_wide_multi_kernel<9>;
    case 10: return (const void *)nr_grid_wide_multi_kernel<10>;
    case 11: return (const void *)nr_grid_wide_multi_kernel<11>;
    case 12: return (const void *)nr_grid_wide_multi_kernel<12>;
    case 13: return (const void *)nr_grid_wide_multi_kernel<13>;
    case 14: return (const void *)nr_grid_wide_multi_kernel<14>;
    case 15: return (const void *)nr_grid_wide_multi_kernel<15>;
    case 16: return (const void *)nr_grid_wide_multi_kernel<16>;
    default: return w4 > NR_WIDE_MAX_W4 ? (const void *)nr_grid_wide_multi_kernel<0> : nullptr;
    }
}
