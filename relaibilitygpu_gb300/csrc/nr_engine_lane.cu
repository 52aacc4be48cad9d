// nr_engine_lane.cu -- one-lane-per-subproblem kernels for undirected simple
// graphs of up to 16 nodes (nr_lane.cuh), one per mask width.
#include "nr_lane2.cuh"

const void *nr_lane_kernel_ptr(int w4)
{
    switch (w4) {
    case 1: return (const void *)nr_lane_kernel<1>;
    case 2: return (const void *)nr_lane_kernel<2>;
    default: return nullptr;
    }
}

const void *nr_lane2_kernel_ptr(int w4, int slots)
{
    if (slots == 2) {
        if (w4 == 1) return (const void *)nr_lane2_kernel<1, 2>;
        if (w4 == 2) return (const void *)nr_lane2_kernel<2, 2>;
    } else if (slots == 4) {
        if (w4 == 1) return (const void *)nr_lane2_kernel<1, 4>;
        if (w4 == 2) return (const void *)nr_lane2_kernel<2, 4>;
    }
    return nullptr;
}
