// nr_mlp.cu -- training and batched inference of the learned scorer (nr_mlp.cuh).
//
// Training runs entirely on the GPU in FP32: a tiled GEMM kernel (16x16
// tiles, optional transposes, fused bias and ReLU), column sums for the bias
// gradients, the binary cross-entropy gradient of the sigmoid output, and an
// Adam step.  Minibatches are gathered on the device from a fixed seeded
// shuffle, so a training run is reproducible.  Inference uses the BF16
// tensor-core routine of nr_mlp.cuh.
#include <algorithm>
#include <cmath>
#include <cstring>
#include <random>
#include <vector>

#include "nr_device.cuh"
#include "nr_mlp.cuh"

#define TILE 16

// C[M][N] = opA(A)[M][K] * opB(B)[K][N] (+ bias[N]) (ReLU), with
// opA(i,k) = tA ? A[k*lda+i] : A[i*lda+k] and opB(k,j) = tB ? B[j*ldb+k] : B[k*ldb+j].
// pre (optional) receives the value before ReLU.
__global__ void nr_mlp_gemm(const float *A, const float *B, float *C, float *pre, const float *bias, int M, int N,
                            int K, int lda, int ldb, int tA, int tB, int relu)
{
    __shared__ float sa[TILE][TILE + 1], sb[TILE][TILE + 1];
    const int tx = threadIdx.x, ty = threadIdx.y;
    const int row = blockIdx.y * TILE + ty, col = blockIdx.x * TILE + tx;
    float acc = 0.f;
    for (int k0 = 0; k0 < K; k0 += TILE) {
        const int ka = k0 + tx, kb = k0 + ty;
        float av = 0.f, bv = 0.f;
        if (row < M && ka < K) av = tA ? A[(size_t)ka * lda + row] : A[(size_t)row * lda + ka];
        if (col < N && kb < K) bv = tB ? B[(size_t)col * ldb + kb] : B[(size_t)kb * ldb + col];
        sa[ty][tx] = av;
        sb[ty][tx] = bv;
        __syncthreads();
#pragma unroll
        for (int k = 0; k < TILE; ++k) acc = fmaf(sa[ty][k], sb[k][tx], acc);
        __syncthreads();
    }
    if (row < M && col < N) {
        if (bias) acc += bias[col];
        if (pre) pre[(size_t)row * N + col] = acc;
        C[(size_t)row * N + col] = relu ? fmaxf(acc, 0.f) : acc;
    }
}

// dZ = dA * (Z > 0)
__global__ void nr_mlp_relu_grad(const float *dA, const float *Z, float *dZ, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dZ[i] = Z[i] > 0.f ? dA[i] : 0.f;
}

// out[j] = sum_i X[i][j] (bias gradients)
__global__ void nr_mlp_colsum(const float *X, float *out, int M, int N)
{
    const int j = blockIdx.x * blockDim.x + threadIdx.x;
    if (j >= N) return;
    float s = 0.f;
    for (int i = 0; i < M; ++i) s += X[(size_t)i * N + j];
    out[j] = s;
}

// output layer: z = A3 w4 + b4; p = sigmoid(z); dz = (p - y) / B; loss terms
__global__ void nr_mlp_head(const float *A3, const float *w4, const float *b4, const float *y, float *dz, float *lossv,
                            int Bn)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= Bn) return;
    float z = b4[0];
    for (int k = 0; k < NR_MLP_H; ++k) z = fmaf(A3[(size_t)i * NR_MLP_H + k], w4[k], z);
    const float p = 1.f / (1.f + expf(-z));
    dz[i] = (p - y[i]) / (float)Bn;
    // binary cross-entropy with logits, written in the stable form
    const float l = fmaxf(z, 0.f) - z * y[i] + log1pf(expf(-fabsf(z)));
    lossv[i] = l;
}

// dA3[i][k] = dz[i] * w4[k]
__global__ void nr_mlp_head_back(const float *dz, const float *w4, float *dA3, int Bn)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Bn * NR_MLP_H) return;
    dA3[t] = dz[t / NR_MLP_H] * w4[t % NR_MLP_H];
}

__global__ void nr_mlp_adam(float *theta, const float *g, float *m, float *v, int n, float lr, float b1, float b2,
                            float eps, float c1, float c2, float wd)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const float gi = g[i] + wd * theta[i];
    const float mi = b1 * m[i] + (1.f - b1) * gi;
    const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
    m[i] = mi;
    v[i] = vi;
    theta[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void nr_mlp_gather(const float *X, const float *y, const int *idx, float *Xb, float *yb, int Bn)
{
    const int t = blockIdx.x * blockDim.x + threadIdx.x;
    if (t >= Bn * NR_MLP_IN) return;
    const int r = t / NR_MLP_IN, k = t % NR_MLP_IN;
    Xb[t] = X[(size_t)idx[r] * NR_MLP_IN + k];
    if (k == 0) yb[r] = y[idx[r]];
}

__global__ void nr_mlp_to_bf16(const float *src, __nv_bfloat16 *dst, int n)
{
    const int i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i < n) dst[i] = __float2bfloat16_rn(src[i]);
}

// batched inference with the tensor-core tile routine; one warp per 16 rows
__global__ void __launch_bounds__(128) nr_mlp_infer_kernel(NrMlpDev M, const float *X, int n, float *y)
{
    __shared__ uint32_t scratch[4][NR_MLP_WARP_WORDS];
    __shared__ float out[4][16];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    const int warps = gridDim.x * (blockDim.x >> 5);
    for (int t = blockIdx.x * (blockDim.x >> 5) + warp; t * 16 < n; t += warps) {
        // 16 rows x 16 features -> bf16 tile (row r, feature k at word r*8 + k/2)
        for (int w = lane; w < 128; w += 32) {
            const int r = w / 8, k = (w % 8) * 2, row = t * 16 + r;
            const float a = row < n ? X[(size_t)row * NR_MLP_IN + k] : 0.f;
            const float b = row < n ? X[(size_t)row * NR_MLP_IN + k + 1] : 0.f;
            scratch[warp][w] = nr_pack_bf16(a, b);
        }
        nr_mlp_warp_infer(M, scratch[warp], out[warp]);
        if (lane < 16 && t * 16 + lane < n) y[t * 16 + lane] = out[warp][lane];
        __syncwarp();
    }
}

// ---------------------------------------------------------------------------
// host side
// ---------------------------------------------------------------------------
namespace {

struct Dev {
    float *p = nullptr;
    size_t n = 0;
};

int dalloc(float **p, size_t n)
{
    if (cudaMalloc(p, n * sizeof(float)) != cudaSuccess) {
        cudaGetLastError();
        *p = nullptr;
        return NR_ERR_NOMEM;
    }
    return NR_OK;
}

void gemm(cudaStream_t s, const float *A, const float *B, float *C, float *pre, const float *bias, int M, int N, int K,
          int lda, int ldb, int tA, int tB, int relu)
{
    dim3 blk(TILE, TILE), grd((N + TILE - 1) / TILE, (M + TILE - 1) / TILE);
    nr_mlp_gemm<<<grd, blk, 0, s>>>(A, B, C, pre, bias, M, N, K, lda, ldb, tA, tB, relu);
}

// workspace for one forward/backward pass on a batch of Bn rows
struct Work {
    float *Z1, *A1, *Z2, *A2, *Z3, *A3, *dz, *loss, *dA, *dZ, *g;
    float *base = nullptr;
    int Bn = 0;
    int init(int b)
    {
        Bn = b;
        const size_t H = NR_MLP_H;
        const size_t total = 6 * b * H + 2 * (size_t)b + 2 * b * H + NR_MLP_PARAMS;
        if (dalloc(&base, total)) return NR_ERR_NOMEM;
        float *q = base;
        Z1 = q; q += b * H; A1 = q; q += b * H; Z2 = q; q += b * H; A2 = q; q += b * H;
        Z3 = q; q += b * H; A3 = q; q += b * H; dz = q; q += b; loss = q; q += b;
        dA = q; q += b * H; dZ = q; q += b * H; g = q;
        return NR_OK;
    }
    ~Work() { if (base) cudaFree(base); }
};

// forward + backward of the batch (X [Bn][16], y [Bn]) with parameters th;
// gradients land in w.g (same layout as th), per-row losses in w.loss.
void fwd_bwd(cudaStream_t s, const float *th, const float *X, const float *y, Work &w)
{
    const int B = w.Bn, H = NR_MLP_H, I = NR_MLP_IN;
    const float *W1 = th + NR_MLP_OFF_W1, *b1 = th + NR_MLP_OFF_B1, *W2 = th + NR_MLP_OFF_W2, *b2 = th + NR_MLP_OFF_B2;
    const float *W3 = th + NR_MLP_OFF_W3, *b3 = th + NR_MLP_OFF_B3, *w4 = th + NR_MLP_OFF_W4, *b4 = th + NR_MLP_OFF_B4;
    float *g = w.g;
    gemm(s, X, W1, w.A1, w.Z1, b1, B, H, I, I, I, 0, 1, 1);
    gemm(s, w.A1, W2, w.A2, w.Z2, b2, B, H, H, H, H, 0, 1, 1);
    gemm(s, w.A2, W3, w.A3, w.Z3, b3, B, H, H, H, H, 0, 1, 1);
    nr_mlp_head<<<(B + 127) / 128, 128, 0, s>>>(w.A3, w4, b4, y, w.dz, w.loss, B);
    // output layer gradients
    gemm(s, w.A3, w.dz, g + NR_MLP_OFF_W4, nullptr, nullptr, H, 1, B, H, 1, 1, 0, 0);    // A3^T dz
    nr_mlp_colsum<<<1, 32, 0, s>>>(w.dz, g + NR_MLP_OFF_B4, B, 1);
    nr_mlp_head_back<<<(B * H + 255) / 256, 256, 0, s>>>(w.dz, w4, w.dA, B);
    // layer 3
    nr_mlp_relu_grad<<<(B * H + 255) / 256, 256, 0, s>>>(w.dA, w.Z3, w.dZ, B * H);
    gemm(s, w.dZ, w.A2, g + NR_MLP_OFF_W3, nullptr, nullptr, H, H, B, H, H, 1, 0, 0);    // dZ3^T A2
    nr_mlp_colsum<<<(H + 127) / 128, 128, 0, s>>>(w.dZ, g + NR_MLP_OFF_B3, B, H);
    gemm(s, w.dZ, W3, w.dA, nullptr, nullptr, B, H, H, H, H, 0, 0, 0);                  // dZ3 W3
    // layer 2
    nr_mlp_relu_grad<<<(B * H + 255) / 256, 256, 0, s>>>(w.dA, w.Z2, w.dZ, B * H);
    gemm(s, w.dZ, w.A1, g + NR_MLP_OFF_W2, nullptr, nullptr, H, H, B, H, H, 1, 0, 0);
    nr_mlp_colsum<<<(H + 127) / 128, 128, 0, s>>>(w.dZ, g + NR_MLP_OFF_B2, B, H);
    gemm(s, w.dZ, W2, w.dA, nullptr, nullptr, B, H, H, H, H, 0, 0, 0);
    // layer 1
    nr_mlp_relu_grad<<<(B * H + 255) / 256, 256, 0, s>>>(w.dA, w.Z1, w.dZ, B * H);
    gemm(s, w.dZ, X, g + NR_MLP_OFF_W1, nullptr, nullptr, H, I, B, H, I, 1, 0, 0);      // dZ1^T X
    nr_mlp_colsum<<<(H + 127) / 128, 128, 0, s>>>(w.dZ, g + NR_MLP_OFF_B1, B, H);
}

}  // namespace

extern "C" int nr_mlp_param_count(void) { return NR_MLP_PARAMS; }

// He-uniform initialisation from a seeded generator (host, deterministic).
extern "C" int nr_mlp_init(float *params, uint64_t seed)
{
    if (!params) return NR_ERR_INVALID;
    std::mt19937_64 rng(seed);
    auto fill = [&](int off, int fan_out, int fan_in) {
        const float b = std::sqrt(6.0f / (float)fan_in);
        std::uniform_real_distribution<float> d(-b, b);
        for (int i = 0; i < fan_out * fan_in; ++i) params[off + i] = d(rng);
    };
    memset(params, 0, sizeof(float) * NR_MLP_PARAMS);
    fill(NR_MLP_OFF_W1, NR_MLP_H, NR_MLP_IN);
    fill(NR_MLP_OFF_W2, NR_MLP_H, NR_MLP_H);
    fill(NR_MLP_OFF_W3, NR_MLP_H, NR_MLP_H);
    fill(NR_MLP_OFF_W4, 1, NR_MLP_H);
    return NR_OK;
}

// One forward + backward pass over the whole set (used to check gradients).
extern "C" int nr_mlp_grad(int device, const float *params, const float *X, const float *y, int n, float *loss,
                           float *grads)
{
    if (!params || !X || !y || n <= 0 || !grads) return NR_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return NR_ERR_CUDA; }
    Work w;
    if (w.init(n)) return NR_ERR_NOMEM;
    float *dth = nullptr, *dX = nullptr, *dy = nullptr;
    if (dalloc(&dth, NR_MLP_PARAMS) || dalloc(&dX, (size_t)n * NR_MLP_IN) || dalloc(&dy, n)) {
        cudaFree(dth); cudaFree(dX); cudaFree(dy);
        return NR_ERR_NOMEM;
    }
    cudaStream_t s = 0;
    cudaMemcpy(dth, params, sizeof(float) * NR_MLP_PARAMS, cudaMemcpyHostToDevice);
    cudaMemcpy(dX, X, sizeof(float) * n * NR_MLP_IN, cudaMemcpyHostToDevice);
    cudaMemcpy(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice);
    fwd_bwd(s, dth, dX, dy, w);
    std::vector<float> lv(n);
    cudaMemcpy(grads, w.g, sizeof(float) * NR_MLP_PARAMS, cudaMemcpyDeviceToHost);
    cudaMemcpy(lv.data(), w.loss, sizeof(float) * n, cudaMemcpyDeviceToHost);
    cudaError_t e = cudaDeviceSynchronize();
    cudaFree(dth); cudaFree(dX); cudaFree(dy);
    if (e != cudaSuccess) { cudaGetLastError(); return NR_ERR_CUDA; }
    double L = 0;
    for (float v : lv) L += v;
    if (loss) *loss = (float)(L / n);
    return NR_OK;
}

// Adam training on (X, y); params holds the initial values on entry and the
// trained ones on return.  loss_per_epoch (optional) gets the mean training loss.
extern "C" int nr_mlp_train(int device, float *params, const float *X, const float *y, int n, int epochs, int batch,
                            float lr, float weight_decay, uint64_t seed, float *loss_per_epoch)
{
    if (!params || !X || !y || n <= 0 || epochs <= 0 || batch <= 0) return NR_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return NR_ERR_CUDA; }
    batch = std::min(batch, n);
    Work w;
    if (w.init(batch)) return NR_ERR_NOMEM;
    float *dth = nullptr, *dm = nullptr, *dv = nullptr, *dX = nullptr, *dy = nullptr, *Xb = nullptr, *yb = nullptr;
    int *didx = nullptr;
    int rc = NR_OK;
    if (dalloc(&dth, NR_MLP_PARAMS) || dalloc(&dm, NR_MLP_PARAMS) || dalloc(&dv, NR_MLP_PARAMS) ||
        dalloc(&dX, (size_t)n * NR_MLP_IN) || dalloc(&dy, n) || dalloc(&Xb, (size_t)batch * NR_MLP_IN) ||
        dalloc(&yb, batch) || cudaMalloc(&didx, sizeof(int) * (size_t)n) != cudaSuccess)
        rc = NR_ERR_NOMEM;
    cudaStream_t s = 0;
    if (rc == NR_OK) {
        cudaMemcpy(dth, params, sizeof(float) * NR_MLP_PARAMS, cudaMemcpyHostToDevice);
        cudaMemset(dm, 0, sizeof(float) * NR_MLP_PARAMS);
        cudaMemset(dv, 0, sizeof(float) * NR_MLP_PARAMS);
        cudaMemcpy(dX, X, sizeof(float) * n * NR_MLP_IN, cudaMemcpyHostToDevice);
        cudaMemcpy(dy, y, sizeof(float) * n, cudaMemcpyHostToDevice);
        std::vector<int> order(n);
        for (int i = 0; i < n; ++i) order[i] = i;
        std::mt19937_64 rng(seed);
        const float b1 = 0.9f, b2 = 0.999f;
        long long step = 0;
        std::vector<float> lv(batch);
        for (int ep = 0; ep < epochs; ++ep) {
            std::shuffle(order.begin(), order.end(), rng);
            cudaMemcpy(didx, order.data(), sizeof(int) * n, cudaMemcpyHostToDevice);
            double ep_loss = 0;
            int nb = 0;
            for (int b0 = 0; b0 + batch <= n; b0 += batch) {
                nr_mlp_gather<<<(batch * NR_MLP_IN + 255) / 256, 256, 0, s>>>(dX, dy, didx + b0, Xb, yb, batch);
                fwd_bwd(s, dth, Xb, yb, w);
                ++step;
                const float c1 = 1.f - std::pow(b1, (float)step), c2 = 1.f - std::pow(b2, (float)step);
                nr_mlp_adam<<<(NR_MLP_PARAMS + 255) / 256, 256, 0, s>>>(dth, w.g, dm, dv, NR_MLP_PARAMS, lr, b1, b2,
                                                                         1e-8f, c1, c2, weight_decay);
                if (loss_per_epoch) {
                    cudaMemcpyAsync(lv.data(), w.loss, sizeof(float) * batch, cudaMemcpyDeviceToHost, s);
                    cudaStreamSynchronize(s);
                    for (float v : lv) ep_loss += v;
                    nb += batch;
                }
            }
            if (loss_per_epoch) loss_per_epoch[ep] = nb ? (float)(ep_loss / nb) : 0.f;
        }
        cudaMemcpy(params, dth, sizeof(float) * NR_MLP_PARAMS, cudaMemcpyDeviceToHost);
        if (cudaDeviceSynchronize() != cudaSuccess) { cudaGetLastError(); rc = NR_ERR_CUDA; }
    }
    cudaFree(dth); cudaFree(dm); cudaFree(dv); cudaFree(dX); cudaFree(dy); cudaFree(Xb); cudaFree(yb); cudaFree(didx);
    return rc;
}

// Upload parameters as the BF16 inference copy; *out receives device pointers.
int nr_mlp_upload(const float *params, void **storage, NrMlpDev *out, cudaStream_t s)
{
    const size_t nw = NR_MLP_PARAMS;
    if (!*storage) {
        if (cudaMalloc(storage, nw * sizeof(float) + nw * sizeof(__nv_bfloat16) + 256) != cudaSuccess) {
            cudaGetLastError();
            return NR_ERR_NOMEM;
        }
    }
    float *f = static_cast<float *>(*storage);
    __nv_bfloat16 *h = reinterpret_cast<__nv_bfloat16 *>(f + nw);
    if (cudaMemcpyAsync(f, params, nw * sizeof(float), cudaMemcpyHostToDevice, s) != cudaSuccess) return NR_ERR_CUDA;
    nr_mlp_to_bf16<<<(int)((nw + 255) / 256), 256, 0, s>>>(f, h, (int)nw);
    out->w1 = h + NR_MLP_OFF_W1;
    out->w2 = h + NR_MLP_OFF_W2;
    out->w3 = h + NR_MLP_OFF_W3;
    out->b1 = f + NR_MLP_OFF_B1;
    out->b2 = f + NR_MLP_OFF_B2;
    out->b3 = f + NR_MLP_OFF_B3;
    out->w4 = f + NR_MLP_OFF_W4;
    out->b4 = params[NR_MLP_OFF_B4];
    return NR_OK;
}

// Batched inference (tensor cores, BF16 weights): y[i] = model(X[i]).
extern "C" int nr_mlp_infer(int device, const float *params, const float *X, int n, float *y)
{
    if (!params || !X || !y || n <= 0) return NR_ERR_INVALID;
    if (cudaSetDevice(device) != cudaSuccess) { cudaGetLastError(); return NR_ERR_CUDA; }
    void *store = nullptr;
    NrMlpDev M;
    float *dX = nullptr, *dy = nullptr;
    int rc = nr_mlp_upload(params, &store, &M, 0);
    if (!rc && (dalloc(&dX, (size_t)n * NR_MLP_IN) || dalloc(&dy, n))) rc = NR_ERR_NOMEM;
    if (!rc) {
        cudaMemcpy(dX, X, sizeof(float) * n * NR_MLP_IN, cudaMemcpyHostToDevice);
        const int tiles = (n + 15) / 16;
        nr_mlp_infer_kernel<<<std::max(1, std::min((tiles + 3) / 4, 4096)), 128>>>(M, dX, n, dy);
        cudaMemcpy(y, dy, sizeof(float) * n, cudaMemcpyDeviceToHost);
        if (cudaDeviceSynchronize() != cudaSuccess) { cudaGetLastError(); rc = NR_ERR_CUDA; }
    }
    cudaFree(store); cudaFree(dX); cudaFree(dy);
    return rc;
}
