// nr_engine_lane.cu -- one-lane-per-subproblem kernels for undirected simple
// graphs of up to 16 nodes (nr_lane.cuh, nr_lane2.cuh), one per mask width, and the
// two-slot kernel with 32-bit rows for 17..32 nodes.
#include "nr_lane2.cuh"
#include "nr_grid_lane.cuh"

const void *nr_lane_kernel_ptr(int w4)
{
    switch (w4) {
    case 1: return (const void *)nr_lane_kernel<1>;
    case 2: return (const void *)nr_lane_kernel<2>;
    default: return nullptr;
    }
}

const void *nr_grid_lane_kernel_ptr(int w4, int row_bits)
{
    if (row_bits == 32) {
        switch (w4) {
        case 1: return (const void *)nr_grid_lane_kernel<1, 32>;
        case 2: return (const void *)nr_grid_lane_kernel<2, 32>;
        case 3: return (const void *)nr_grid_lane_kernel<3, 32>;
        case 4: return (const void *)nr_grid_lane_kernel<4, 32>;
        case 5: return (const void *)nr_grid_lane_kernel<5, 32>;
        case 6: return (const void *)nr_grid_lane_kernel<6, 32>;
        case 7: return (const void *)nr_grid_lane_kernel<7, 32>;
        case 8: return (const void *)nr_grid_lane_kernel<8, 32>;
        default: return nullptr;
        }
    }
    switch (w4) {
    case 1: return (const void *)nr_grid_lane_kernel<1>;
    case 2: return (const void *)nr_grid_lane_kernel<2>;
    default: return nullptr;
    }
}

const void *nr_lane2_kernel_ptr(int w4, int slots, int row_bits)
{
    if (row_bits == 32) {                   // 17..32 nodes: two slots a warp
        if (slots != 2) return nullptr;
        switch (w4) {
        case 1: return (const void *)nr_lane2_kernel<1, 2, 32>;
        case 2: return (const void *)nr_lane2_kernel<2, 2, 32>;
        case 3: return (const void *)nr_lane2_kernel<3, 2, 32>;
        case 4: return (const void *)nr_lane2_kernel<4, 2, 32>;
        case 5: return (const void *)nr_lane2_kernel<5, 2, 32>;
        case 6: return (const void *)nr_lane2_kernel<6, 2, 32>;
        case 7: return (const void *)nr_lane2_kernel<7, 2, 32>;
        case 8: return (const void *)nr_lane2_kernel<8, 2, 32>;
        default: return nullptr;
        }
    }
    if (slots == 2) {
        if (w4 == 1) return (const void *)nr_lane2_kernel<1, 2>;
        if (w4 == 2) return (const void *)nr_lane2_kernel<2, 2>;
    } else if (slots == 4) {
        if (w4 == 1) return (const void *)nr_lane2_kernel<1, 4>;
        if (w4 == 2) return (const void *)nr_lane2_kernel<2, 4>;
    }
    return nullptr;
}
