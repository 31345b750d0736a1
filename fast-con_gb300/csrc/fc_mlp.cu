// fc_mlp.cu -- training of the learned schedule's MLP on the GPU, and the
// entry points that install its weights.
//
// Network (fc_sched.cuh): 12 features -> 32 ReLU -> 32 ReLU -> 7 logits in
// three heads: side (logits 0-1), direction (2-3), expansion variant (4-6).
// Loss: softmax cross-entropy per head, summed over the heads that carry a
// label (label -1 = none), each head's term multiplied by the sample's weight
// for that head (1 when no weights are given; training uses the cost of a
// wrong choice), averaged over the samples of the batch.
//
// Kernels:
//   k_mlp_grad   one warp per sample: lane j owns hidden unit j in the
//                forward pass (like the inference warp in the traversal
//                loop) and in the backward pass; gradients are accumulated in
//                shared memory and added to the global gradient once per CTA.
//   k_adam       Adam update of the 1,703 parameters (Kingma & Ba, 2015).
// softmax uses CUDA's expf / logf.
#include <cmath>
#include <cfloat>
#include <cstring>
#include <vector>

#include "fastcon.h"
#include "fc_engine.h"
#include "fc_sched.cuh"

namespace fc {

constexpr int MLP_BLOCK = 256;

__global__ void __launch_bounds__(MLP_BLOCK) k_mlp_grad(const float *__restrict__ X,
                                                        const int32_t *__restrict__ Y,
                                                        const float *__restrict__ SW, int n,
                                                        const float *__restrict__ W,
                                                        float *__restrict__ grad, float *loss_sum,
                                                        float scale)
{
    __shared__ float g[MLP_PARAMS];
    __shared__ float wl[MLP_BLOCK / 32];
    for (int i = threadIdx.x; i < MLP_PARAMS; i += MLP_BLOCK) g[i] = 0.f;
    __syncthreads();
    const int lane = threadIdx.x & 31, wid = threadIdx.x >> 5;
    const int warps = (gridDim.x * MLP_BLOCK) >> 5;
    float loss_acc = 0.f;
    for (int smp = blockIdx.x * (MLP_BLOCK / 32) + wid; smp < n; smp += warps) {
        const float *x = X + (size_t)smp * MLP_IN;
        const int32_t *y = Y + (size_t)smp * 3;
        // forward
        float a1 = W[MLP_B1 + lane];
        for (int i = 0; i < MLP_IN; ++i) a1 += W[MLP_W1 + lane * MLP_IN + i] * x[i];
        const float h1 = a1 > 0.f ? a1 : 0.f;
        float a2 = W[MLP_B2 + lane];
        for (int k = 0; k < MLP_H; ++k) a2 += W[MLP_W2 + lane * MLP_H + k] * __shfl_sync(0xffffffffu, h1, k);
        const float h2 = a2 > 0.f ? a2 : 0.f;
        float z[MLP_OUT];
        for (int o = 0; o < MLP_OUT; ++o) {
            float v = W[MLP_W3 + o * MLP_H + lane] * h2;
            for (int s = 16; s > 0; s >>= 1) v += __shfl_xor_sync(0xffffffffu, v, s);
            z[o] = v + W[MLP_B3 + o];
        }
        // softmax cross-entropy per labelled head; dz = (p - onehot) * scale
        float dz[MLP_OUT];
        const int lo[3] = {0, 2, 4}, len[3] = {2, 2, 3};
        float L = 0.f;
        for (int h = 0; h < 3; ++h) {
            const int label = y[h];
            const float wgt = SW ? SW[(size_t)smp * 3 + h] : 1.f;
            float mx = z[lo[h]];
            for (int k = 1; k < len[h]; ++k) mx = fmaxf(mx, z[lo[h] + k]);
            float se = 0.f;
            for (int k = 0; k < len[h]; ++k) se += expf(z[lo[h] + k] - mx);
            for (int k = 0; k < len[h]; ++k) {
                if (label < 0) {
                    dz[lo[h] + k] = 0.f;
                } else {
                    const float p = expf(z[lo[h] + k] - mx) / se;
                    dz[lo[h] + k] = (p - (k == label ? 1.f : 0.f)) * scale * wgt;
                }
            }
            if (label >= 0) L += wgt * (logf(se) + mx - z[lo[h] + label]);
        }
        loss_acc += L;
        // backward
        float dh2 = 0.f;
        for (int o = 0; o < MLP_OUT; ++o) {
            atomicAdd(&g[MLP_W3 + o * MLP_H + lane], dz[o] * h2);
            dh2 += W[MLP_W3 + o * MLP_H + lane] * dz[o];
        }
        if (lane < MLP_OUT) atomicAdd(&g[MLP_B3 + lane], dz[lane]);
        const float da2 = h2 > 0.f ? dh2 : 0.f;
        for (int k = 0; k < MLP_H; ++k)
            atomicAdd(&g[MLP_W2 + lane * MLP_H + k], da2 * __shfl_sync(0xffffffffu, h1, k));
        atomicAdd(&g[MLP_B2 + lane], da2);
        // dh1[lane] = sum_j W2[j][lane] * da2[j]
        float dh1 = 0.f;
        for (int j = 0; j < MLP_H; ++j) dh1 += W[MLP_W2 + j * MLP_H + lane] * __shfl_sync(0xffffffffu, da2, j);
        const float da1 = h1 > 0.f ? dh1 : 0.f;
        for (int i = 0; i < MLP_IN; ++i) atomicAdd(&g[MLP_W1 + lane * MLP_IN + i], da1 * x[i]);
        atomicAdd(&g[MLP_B1 + lane], da1);
    }
    if (lane == 0) wl[wid] = loss_acc;
    __syncthreads();
    for (int i = threadIdx.x; i < MLP_PARAMS; i += MLP_BLOCK)
        if (g[i] != 0.f) atomicAdd(&grad[i], g[i]);
    if (threadIdx.x == 0) {
        float s = 0.f;
        for (int w = 0; w < MLP_BLOCK / 32; ++w) s += wl[w];
        atomicAdd(loss_sum, s);
    }
}

__global__ void k_adam(float *W, const float *grad, float *m, float *v, int n, float lr, float b1,
                       float b2, float eps, float c1, float c2)
{
    for (int i = blockIdx.x * blockDim.x + threadIdx.x; i < n; i += gridDim.x * blockDim.x) {
        const float gi = grad[i];
        const float mi = b1 * m[i] + (1.f - b1) * gi;
        const float vi = b2 * v[i] + (1.f - b2) * gi * gi;
        m[i] = mi;
        v[i] = vi;
        W[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
    }
}

static int mlp_grid(int n)
{
    int g = (n + MLP_BLOCK / 32 - 1) / (MLP_BLOCK / 32);
    if (g > 152 * 4) g = 152 * 4;
    return g < 1 ? 1 : g;
}

// n = MLP_PARAMS (no feature box: the network is always consulted) or
// MLP_STORE (parameters followed by the box lo[12], hi[12]).
int set_mlp_weights(DevCtx *c, const float *w, int n)
{
    static_assert(sizeof(c->h_mlp) == sizeof(float) * MLP_STORE, "weight store size");
    float h[MLP_STORE];
    std::memcpy(h, w, sizeof(float) * MLP_PARAMS);
    for (int i = 0; i < MLP_IN; ++i) {
        h[MLP_BOX + i] = n == MLP_STORE ? w[MLP_BOX + i] : -FLT_MAX;
        h[MLP_BOX + MLP_IN + i] = n == MLP_STORE ? w[MLP_BOX + MLP_IN + i] : FLT_MAX;
    }
    if (!c->d_mlp) FC_CUDA_TRY(cudaMalloc(&c->d_mlp, sizeof(float) * MLP_STORE));
    FC_CUDA_TRY(cudaMemcpy(c->d_mlp, h, sizeof(float) * MLP_STORE, cudaMemcpyHostToDevice));
    FC_CUDA_TRY(cudaDeviceSynchronize());  // read by kernels on non-blocking streams
    std::memcpy(c->h_mlp, h, sizeof(float) * MLP_STORE);
    c->mlp_ready = 1;
    return FC_OK;
}

}  // namespace fc

using namespace fc;

extern "C" int fc_sched_set_weights(const float *w, int32_t n)
{
    if (!w || (n != MLP_PARAMS && n != MLP_STORE)) {
        set_error("fc_sched_set_weights: expected %d or %d floats", MLP_PARAMS, MLP_STORE);
        return FC_ERR_INVALID;
    }
    int rc = FC_OK;
    DevCtx *c = get_ctx(&rc);
    if (!c) return rc;
    std::lock_guard<std::mutex> lk(c->mu);
    return set_mlp_weights(c, w, n);
}

extern "C" int fc_sched_get_weights(float *w, int32_t n)
{
    if (!w || (n != MLP_PARAMS && n != MLP_STORE)) return FC_ERR_INVALID;
    int rc = FC_OK;
    DevCtx *c = get_ctx(&rc);
    if (!c) return rc;
    std::lock_guard<std::mutex> lk(c->mu);
    if (!c->mlp_ready) {
        set_error("no weights loaded");
        return FC_ERR_INVALID;
    }
    std::memcpy(w, c->h_mlp, sizeof(float) * (size_t)n);
    return FC_OK;
}

// One forward/backward pass over (X, Y); grad receives the mean gradient.
extern "C" int fc_mlp_loss_grad(const float *X, const int32_t *Y, const float *SW, int32_t n,
                                const float *w, float *grad, float *loss)
{
    if (!X || !Y || !w || !grad || !loss || n <= 0) return FC_ERR_INVALID;
    int rc = FC_OK;
    DevCtx *c = get_ctx(&rc);
    if (!c) return rc;
    float *dX = nullptr, *dW = nullptr, *dG = nullptr, *dL = nullptr, *dS = nullptr;
    int32_t *dY = nullptr;
    if (SW) {
        FC_CUDA_TRY(cudaMalloc(&dS, sizeof(float) * (size_t)n * 3));
        FC_CUDA_TRY(cudaMemcpy(dS, SW, sizeof(float) * (size_t)n * 3, cudaMemcpyHostToDevice));
    }
    FC_CUDA_TRY(cudaMalloc(&dX, sizeof(float) * (size_t)n * MLP_IN));
    FC_CUDA_TRY(cudaMalloc(&dY, sizeof(int32_t) * (size_t)n * 3));
    FC_CUDA_TRY(cudaMalloc(&dW, sizeof(float) * MLP_PARAMS));
    FC_CUDA_TRY(cudaMalloc(&dG, sizeof(float) * (MLP_PARAMS + 1)));
    dL = dG + MLP_PARAMS;
    FC_CUDA_TRY(cudaMemcpy(dX, X, sizeof(float) * (size_t)n * MLP_IN, cudaMemcpyHostToDevice));
    FC_CUDA_TRY(cudaMemcpy(dY, Y, sizeof(int32_t) * (size_t)n * 3, cudaMemcpyHostToDevice));
    FC_CUDA_TRY(cudaMemcpy(dW, w, sizeof(float) * MLP_PARAMS, cudaMemcpyHostToDevice));
    FC_CUDA_TRY(cudaMemset(dG, 0, sizeof(float) * (MLP_PARAMS + 1)));
    k_mlp_grad<<<mlp_grid(n), MLP_BLOCK>>>(dX, dY, dS, n, dW, dG, dL, 1.f / (float)n);
    FC_CUDA_TRY(cudaGetLastError());
    FC_CUDA_TRY(cudaMemcpy(grad, dG, sizeof(float) * MLP_PARAMS, cudaMemcpyDeviceToHost));
    float ls = 0;
    FC_CUDA_TRY(cudaMemcpy(&ls, dL, sizeof(float), cudaMemcpyDeviceToHost));
    *loss = ls / (float)n;
    cudaFree(dX);
    cudaFree(dY);
    cudaFree(dW);
    cudaFree(dG);
    cudaFree(dS);
    return FC_OK;
}

// Mini-batch Adam training on the GPU.  w_inout holds the initial weights and
// receives the trained ones; loss_curve (nullable) gets the mean training loss
// of each epoch.  Samples are visited in a fixed order (the caller shuffles).
extern "C" int fc_mlp_train(const float *X, const int32_t *Y, const float *SW, int32_t n,
                            int32_t epochs, int32_t batch, float lr, float *w_inout,
                            float *loss_curve)
{
    if (!X || !Y || !w_inout || n <= 0 || epochs <= 0 || batch <= 0) return FC_ERR_INVALID;
    int rc = FC_OK;
    DevCtx *c = get_ctx(&rc);
    if (!c) return rc;
    float *dX = nullptr, *dW = nullptr, *dG = nullptr, *dM = nullptr, *dV = nullptr, *dS = nullptr;
    int32_t *dY = nullptr;
    if (SW) {
        FC_CUDA_TRY(cudaMalloc(&dS, sizeof(float) * (size_t)n * 3));
        FC_CUDA_TRY(cudaMemcpy(dS, SW, sizeof(float) * (size_t)n * 3, cudaMemcpyHostToDevice));
    }
    FC_CUDA_TRY(cudaMalloc(&dX, sizeof(float) * (size_t)n * MLP_IN));
    FC_CUDA_TRY(cudaMalloc(&dY, sizeof(int32_t) * (size_t)n * 3));
    FC_CUDA_TRY(cudaMalloc(&dW, sizeof(float) * MLP_PARAMS * 4 + sizeof(float) * 4));
    dG = dW + MLP_PARAMS;
    dM = dG + MLP_PARAMS;
    dV = dM + MLP_PARAMS;
    float *dL = dV + MLP_PARAMS;
    FC_CUDA_TRY(cudaMemcpy(dX, X, sizeof(float) * (size_t)n * MLP_IN, cudaMemcpyHostToDevice));
    FC_CUDA_TRY(cudaMemcpy(dY, Y, sizeof(int32_t) * (size_t)n * 3, cudaMemcpyHostToDevice));
    FC_CUDA_TRY(cudaMemcpy(dW, w_inout, sizeof(float) * MLP_PARAMS, cudaMemcpyHostToDevice));
    FC_CUDA_TRY(cudaMemset(dM, 0, sizeof(float) * MLP_PARAMS * 2));
    const float b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
    double p1 = 1.0, p2 = 1.0;
    for (int ep = 0; ep < epochs; ++ep) {
        FC_CUDA_TRY(cudaMemset(dL, 0, sizeof(float)));
        for (int b0 = 0; b0 < n; b0 += batch) {
            const int nb = n - b0 < batch ? n - b0 : batch;
            FC_CUDA_TRY(cudaMemset(dG, 0, sizeof(float) * MLP_PARAMS));
            k_mlp_grad<<<mlp_grid(nb), MLP_BLOCK>>>(dX + (size_t)b0 * MLP_IN, dY + (size_t)b0 * 3,
                                                    dS ? dS + (size_t)b0 * 3 : nullptr, nb, dW, dG,
                                                    dL, 1.f / (float)nb);
            p1 *= b1;
            p2 *= b2;
            k_adam<<<(MLP_PARAMS + 255) / 256, 256>>>(dW, dG, dM, dV, MLP_PARAMS, lr, b1, b2, eps,
                                                      (float)(1.0 - p1), (float)(1.0 - p2));
        }
        FC_CUDA_TRY(cudaGetLastError());
        if (loss_curve) {
            float ls = 0;
            FC_CUDA_TRY(cudaMemcpy(&ls, dL, sizeof(float), cudaMemcpyDeviceToHost));
            loss_curve[ep] = ls / (float)n;
        }
    }
    FC_CUDA_TRY(cudaMemcpy(w_inout, dW, sizeof(float) * MLP_PARAMS, cudaMemcpyDeviceToHost));
    cudaFree(dX);
    cudaFree(dY);
    cudaFree(dW);
    cudaFree(dS);
    return FC_OK;
}
