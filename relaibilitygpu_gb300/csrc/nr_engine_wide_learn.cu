// nr_engine_wide_learn.cu -- the bucketed whole-GPU kernel with the learned branch order
// (graphs with 33..16384 nodes), one per mask width; its own translation unit keeps the build
// parallel.
#include "nr_wide.cuh"

const void *nr_bucket_wide_learn_kernel_ptr(int w4)
{
    switch (w4) {
    case 1: return (const void *)nr_bucket_wide_kernel<1, true>;
    case 2: return (const void *)nr_bucket_wide_kernel<2, true>;
    case 3: return (const void *)nr_bucket_wide_kernel<3, true>;
    case 4: return (const void *)nr_bucket_wide_kernel<4, true>;
    case 5: return (const void *)nr_bucket_wide_kernel<5, true>;
    case 6: return (const void *)nr_bucket_wide_kernel<6, true>;
    case 7: return (const void *)nr_bucket_wide_kernel<7, true>;
    case 8: return (const void *)nr_bucket_wide_kernel<8, true>;
    case 9: return (const void *)nr_bucket_wide_kernel<9, true>;
    case 10: return (const void *)nr_bucket_wide_kernel<10, true>;
    case 11: return (const void *)nr_bucket_wide_kernel<11, true>;
    case 12: return (const void *)nr_bucket_wide_kernel<12, true>;
    case 13: return (const void *)nr_bucket_wide_kernel<13, true>;
    case 14: return (const void *)nr_bucket_wide_kernel<14, true>;
    case 15: return (const void *)nr_bucket_wide_kernel<15, true>;
    case 16: return (const void *)nr_bucket_wide_kernel<16, true>;
    default: return w4 > NR_WIDE_MAX_W4 ? (const void *)nr_bucket_wide_kernel<0, true> : nullptr;
    }
}
