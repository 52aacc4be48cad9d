// nr_engine_wide.cu -- kernels for graphs with 33..16384 nodes: mask blocks 1..16 compiled in,
// wider masks (up to 65535 edges) in the runtime-width instantiation W4 = 0.
#include "nr_wide.cuh"

const void *nr_grid_wide_kernel_ptr(int w4)
{
    switch (w4) {
    case 1: return (const void *)nr_grid_wide_kernel<1>;
    case 2: return (const void *)nr_grid_wide_kernel<2>;
    case 3: return (const void *)nr_grid_wide_kernel<3>;
    case 4: return (const void *)nr_grid_wide_kernel<4>;
    case 5: return (const void *)nr_grid_wide_kernel<5>;
    case 6: return (const void *)nr_grid_wide_kernel<6>;
    case 7: return (const void *)nr_grid_wide_kernel<7>;
    case 8: return (const void *)nr_grid_wide_kernel<8>;
    case 9: return (const void *)nr_grid_wide_kernel<9>;
    case 10: return (const void *)nr_grid_wide_kernel<10>;
    case 11: return (const void *)nr_grid_wide_kernel<11>;
    case 12: return (const void *)nr_grid_wide_kernel<12>;
    case 13: return (const void *)nr_grid_wide_kernel<13>;
    case 14: return (const void *)nr_grid_wide_kernel<14>;
    case 15: return (const void *)nr_grid_wide_kernel<15>;
    case 16: return (const void *)nr_grid_wide_kernel<16>;
    default: return w4 > NR_WIDE_MAX_W4 ? (const void *)nr_grid_wide_kernel<0> : nullptr;
    }
}

const void *nr_bucket_wide_kernel_ptr(int w4)
{
    switch (w4) {
    case 1: return (const void *)nr_bucket_wide_kernel<1>;
    case 2: return (const void *)nr_bucket_wide_kernel<2>;
    case 3: return (const void *)nr_bucket_wide_kernel<3>;
    case 4: return (const void *)nr_bucket_wide_kernel<4>;
    case 5: return (const void *)nr_bucket_wide_kernel<5>;
    case 6: return (const void *)nr_bucket_wide_kernel<6>;
    case 7: return (const void *)nr_bucket_wide_kernel<7>;
    case 8: return (const void *)nr_bucket_wide_kernel<8>;
    case 9: return (const void *)nr_bucket_wide_kernel<9>;
    case 10: return (const void *)nr_bucket_wide_kernel<10>;
    case 11: return (const void *)nr_bucket_wide_kernel<11>;
    case 12: return (const void *)nr_bucket_wide_kernel<12>;
    case 13: return (const void *)nr_bucket_wide_kernel<13>;
    case 14: return (const void *)nr_bucket_wide_kernel<14>;
    case 15: return (const void *)nr_bucket_wide_kernel<15>;
    case 16: return (const void *)nr_bucket_wide_kernel<16>;
    default: return w4 > NR_WIDE_MAX_W4 ? (const void *)nr_bucket_wide_kernel<0> : nullptr;
    }
}
