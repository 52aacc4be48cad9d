// nr_engine_wide_lanes.cu -- the bucketed whole-GPU queue with one lane per subproblem
// (nr_bucket_wide_kernel<W4, false, true>), one instantiation per compiled mask width.
#include "nr_wide.cuh"

const void *nr_bucket_wide_lanes_kernel_ptr(int w4)
{
    switch (w4) {
    case 1: return (const void *)nr_bucket_wide_kernel<1, false, true>;
    case 2: return (const void *)nr_bucket_wide_kernel<2, false, true>;
    case 3: return (const void *)nr_bucket_wide_kernel<3, false, true>;
    case 4: return (const void *)nr_bucket_wide_kernel<4, false, true>;
    case 5: return (const void *)nr_bucket_wide_kernel<5, false, true>;
    case 6: return (const void *)nr_bucket_wide_kernel<6, false, true>;
    case 7: return (const void *)nr_bucket_wide_kernel<7, false, true>;
    case 8: return (const void *)nr_bucket_wide_kernel<8, false, true>;
    case 9: return (const void *)nr_bucket_wide_kernel<9, false, true>;
    case 10: return (const void *)nr_bucket_wide_kernel<10, false, true>;
    case 11: return (const void *)nr_bucket_wide_kernel<11, false, true>;
    case 12: return (const void *)nr_bucket_wide_kernel<12, false, true>;
    case 13: return (const void *)nr_bucket_wide_kernel<13, false, true>;
    case 14: return (const void *)nr_bucket_wide_kernel<14, false, true>;
    case 15: return (const void *)nr_bucket_wide_kernel<15, false, true>;
    case 16: return (const void *)nr_bucket_wide_kernel<16, false, true>;
    default: return nullptr;
    }
}
