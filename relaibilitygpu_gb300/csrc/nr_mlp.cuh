// nr_mlp.cuh -- the learned scorer: an MLP 16 -> 128 -> 128 -> 128 -> 1
// (ReLU, sigmoid output) that estimates a subproblem's residual reliability
// from cheap mask features.  It only sets the priority (bucket key) of a
// subproblem in the learned order; masses, R and ESP never depend on it.
//
// Inference (nr_mlp_warp_infer): BF16 weights, FP32 accumulation, tensor
// cores through warp-level mma.sync.m16n8k16 on tiles of 16 subproblems.
// The engine scores the children of one warp step at a time (1-32 rows), a
// latency-bound use where one warp's own MMAs beat any CTA-wide handoff.
// Training: FP32 master weights, hand-written tiled GEMM, bias/ReLU and Adam
// kernels (nr_mlp.cu).
#pragma once

#include <cuda_bf16.h>

#include "nr_internal.h"

#define NR_MLP_IN 16
#define NR_MLP_H 128
// flat FP32 parameter layout: W1[H][IN] b1[H] W2[H][H] b2[H] W3[H][H] b3[H] w4[H] b4
#define NR_MLP_OFF_W1 0
#define NR_MLP_OFF_B1 (NR_MLP_OFF_W1 + NR_MLP_H * NR_MLP_IN)
#define NR_MLP_OFF_W2 (NR_MLP_OFF_B1 + NR_MLP_H)
#define NR_MLP_OFF_B2 (NR_MLP_OFF_W2 + NR_MLP_H * NR_MLP_H)
#define NR_MLP_OFF_W3 (NR_MLP_OFF_B2 + NR_MLP_H)
#define NR_MLP_OFF_B3 (NR_MLP_OFF_W3 + NR_MLP_H * NR_MLP_H)
#define NR_MLP_OFF_W4 (NR_MLP_OFF_B3 + NR_MLP_H)
#define NR_MLP_OFF_B4 (NR_MLP_OFF_W4 + NR_MLP_H)
#define NR_MLP_PARAMS (NR_MLP_OFF_B4 + 1)

// Inference copy on the device: BF16 weight matrices (row-major [out][in]),
// FP32 biases and output layer.
struct NrMlpDev {
    const __nv_bfloat16 *w1, *w2, *w3;
    const float *b1, *b2, *b3, *w4;
    float b4;
};

// per-warp shared scratch of nr_mlp_warp_infer, in 32-bit words:
// input tile 16x16 bf16 (128 words) + two activation tiles 16x128 bf16 (2 x 1024 words)
#define NR_MLP_WARP_WORDS (128 + 2 * 1024)

__device__ __forceinline__ uint32_t nr_pack_bf16(float lo, float hi)
{
    const __nv_bfloat162 v = __floats2bfloat162_rn(lo, hi);   // .x = lo (low half), .y = hi
    return *reinterpret_cast<const uint32_t *>(&v);
}

__device__ __forceinline__ void nr_mma_bf16(float (&d)[4], const uint32_t (&a)[4], uint32_t b0, uint32_t b1)
{
    asm volatile(
        "mma.sync.aligned.m16n8k16.row.col.f32.bf16.bf16.f32 {%0,%1,%2,%3}, {%4,%5,%6,%7}, {%8,%9}, "
        "{%0,%1,%2,%3};\n"
        : "+f"(d[0]), "+f"(d[1]), "+f"(d[2]), "+f"(d[3])
        : "r"(a[0]), "r"(a[1]), "r"(a[2]), "r"(a[3]), "r"(b0), "r"(b1));
}

// One dense layer on a 16-row tile: out[16][128] = relu(in[16][K] W^T + b), with
// in and out as row-major bf16 tiles in shared memory (32-bit words, K/2 and
// 64 words per row).  W is [128][K] bf16 in global memory (read through L1).
template <int K>
__device__ __forceinline__ void nr_mlp_layer(const uint32_t *in, uint32_t *out, const __nv_bfloat16 *W,
                                             const float *bias)
{
    const int lane = threadIdx.x & 31;
    const int g = lane >> 2, c = (lane & 3) * 2;
    const uint32_t *Wu = reinterpret_cast<const uint32_t *>(W);
#pragma unroll
    for (int half = 0; half < 2; ++half) {
        float acc[8][4];
#pragma unroll
        for (int j = 0; j < 8; ++j) acc[j][0] = acc[j][1] = acc[j][2] = acc[j][3] = 0.f;
#pragma unroll
        for (int kt = 0; kt < K / 16; ++kt) {
            uint32_t a[4];
            a[0] = in[g * (K / 2) + kt * 8 + c / 2];
            a[1] = in[(g + 8) * (K / 2) + kt * 8 + c / 2];
            a[2] = in[g * (K / 2) + kt * 8 + 4 + c / 2];
            a[3] = in[(g + 8) * (K / 2) + kt * 8 + 4 + c / 2];
#pragma unroll
            for (int j = 0; j < 8; ++j) {
                const int o = half * 64 + j * 8 + g;              // output row of W for this thread
                const uint32_t b0 = __ldg(Wu + o * (K / 2) + kt * 8 + c / 2);
                const uint32_t b1 = __ldg(Wu + o * (K / 2) + kt * 8 + 4 + c / 2);
                nr_mma_bf16(acc[j], a, b0, b1);
            }
        }
#pragma unroll
        for (int j = 0; j < 8; ++j) {
            const int col = half * 64 + j * 8 + c;
            const float bb0 = __ldg(bias + col), bb1 = __ldg(bias + col + 1);
            out[g * 64 + col / 2] = nr_pack_bf16(fmaxf(acc[j][0] + bb0, 0.f), fmaxf(acc[j][1] + bb1, 0.f));
            out[(g + 8) * 64 + col / 2] = nr_pack_bf16(fmaxf(acc[j][2] + bb0, 0.f), fmaxf(acc[j][3] + bb1, 0.f));
        }
    }
    __syncwarp();
}

__device__ __forceinline__ void nr_mlp_warp_infer(const NrMlpDev &M, uint32_t *scratch, float *y);

// Score one row per lane that has one (16-row tiles, the lanes' rows in lane order); returns the
// lane's output (0 for a lane without a row).  Rows of a last, partial tile beyond the lanes'
// keep older features: an output row depends only on its own input row, and those are not read.
// All 32 lanes must call it.
__device__ __forceinline__ float nr_mlp_score_lanes(const NrMlpDev &M, uint32_t *scratch, float *y, bool has,
                                                    const float (&f)[NR_MLP_IN])
{
    const int lane = threadIdx.x & 31;
    const unsigned m = __ballot_sync(0xffffffffu, has);
    const int cnt = __popc(m), rank = __popc(m & ((1u << lane) - 1u));
    float out = 0.f;
    for (int t = 0; t * 16 < cnt; ++t) {
        if (has && rank / 16 == t) {
#pragma unroll
            for (int k = 0; k < NR_MLP_IN / 2; ++k) scratch[(rank % 16) * 8 + k] = nr_pack_bf16(f[2 * k], f[2 * k + 1]);
        }
        nr_mlp_warp_infer(M, scratch, y);
        if (has && rank / 16 == t) out = y[rank % 16];
        __syncwarp();
    }
    return out;
}

// Score a 16-row tile whose BF16 features are already in scratch[0..127]
// (row r, feature k at word r*8 + k/2).  Writes sigmoid outputs to y[16]
// (shared memory).  All 32 lanes must call it.
__device__ __forceinline__ void nr_mlp_warp_infer(const NrMlpDev &M, uint32_t *scratch, float *y)
{
    const int lane = threadIdx.x & 31;
    uint32_t *x = scratch, *h1 = scratch + 128, *h2 = scratch + 128 + 1024;
    __syncwarp();
    nr_mlp_layer<NR_MLP_IN>(x, h1, M.w1, M.b1);
    nr_mlp_layer<NR_MLP_H>(h1, h2, M.w2, M.b2);
    nr_mlp_layer<NR_MLP_H>(h2, h1, M.w3, M.b3);
    // output layer in FP32: two lanes per row, 64 hidden units each
    const int r = lane >> 1, part = lane & 1;
    float s = 0.f;
    const __nv_bfloat162 *hr = reinterpret_cast<const __nv_bfloat162 *>(h1 + r * 64 + part * 32);
#pragma unroll 8
    for (int k = 0; k < 32; ++k) {
        const float2 v = __bfloat1622float2(hr[k]);
        s = fmaf(v.x, __ldg(M.w4 + part * 64 + 2 * k), s);
        s = fmaf(v.y, __ldg(M.w4 + part * 64 + 2 * k + 1), s);
    }
    s += __shfl_xor_sync(0xffffffffu, s, 1);
    if (part == 0) y[r] = 1.f / (1.f + __expf(-(s + M.b4)));
    __syncwarp();
}
