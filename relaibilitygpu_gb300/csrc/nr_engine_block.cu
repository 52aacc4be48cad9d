// nr_engine_block.cu -- the block kernels, one instantiation per row width and mask width: the
// instances the two-slot lane kernel hands over (nr_block_lane.cuh), and a batch's graphs of
// 33..64 nodes (nr_block64.cuh).
#include "nr_block64.cuh"

const void *nr_block_lane_kernel_ptr(int w4, int row_bits)
{
    if (row_bits == 32) {
        switch (w4) {
        case 1: return (const void *)nr_block_lane_kernel<1, 32>;
        case 2: return (const void *)nr_block_lane_kernel<2, 32>;
        case 3: return (const void *)nr_block_lane_kernel<3, 32>;
        case 4: return (const void *)nr_block_lane_kernel<4, 32>;
        case 5: return (const void *)nr_block_lane_kernel<5, 32>;
        case 6: return (const void *)nr_block_lane_kernel<6, 32>;
        case 7: return (const void *)nr_block_lane_kernel<7, 32>;
        case 8: return (const void *)nr_block_lane_kernel<8, 32>;
        default: return nullptr;
        }
    }
    switch (w4) {
    case 1: return (const void *)nr_block_lane_kernel<1, 16>;
    case 2: return (const void *)nr_block_lane_kernel<2, 16>;
    default: return nullptr;
    }
}

const void *nr_block64_kernel_ptr(int w4)
{
    switch (w4) {
    case 1: return (const void *)nr_block64_kernel<1>;
    case 2: return (const void *)nr_block64_kernel<2>;
    case 3: return (const void *)nr_block64_kernel<3>;
    case 4: return (const void *)nr_block64_kernel<4>;
    default: return nullptr;
    }
}
