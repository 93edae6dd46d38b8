// cost_model.cu -- the learned scheduler: a small MLP that predicts a query's work from cheap features, trained on
// the device by the kernels below (forward, backward, Adam), and used to order the persistent kernel's root tasks
// largest-first.
//
// Why: the persistent kernel claims root tasks in order and appends child tasks behind them.  A batch ends when its
// longest remaining chain of tasks ends, so queries that will descend (a root task, then one or more child tasks)
// and long queries should start first.  Their work is not known before the query runs: a query drawn from a user
// bin counts fully at the root and descends, a query of random values stops early at the root.  The features
// (query.cuh, k_query_features: length, relative threshold, and the root's counts over the first few values) let the
// model tell them apart.  Only the order of the tasks changes, so results stay exact.
//
// Model: 6 features -> 32 ReLU -> 32 ReLU -> 1, trained by full-batch Adam on the mean squared error of
// log(1 + executed value visits), the per-query work the query kernel records (hibf_gpu_agent_set_work_out_d).
// Parameters, flat float32: W1[32][6], b1[32], W2[32][32], b2[32], w3[32], b3.

#include <algorithm>
#include <cmath>
#include <cub/cub.cuh>
#include <vector>

#include "../../include/hibf_gb300_synthetic.h"
#include "common.hpp"

namespace hibf_gb300
{
int sm_count();

namespace
{

constexpr int kF = 6;
constexpr int kH = 32;
constexpr int oW1 = 0;
constexpr int oB1 = oW1 + kH * kF;
constexpr int oW2 = oB1 + kH;
constexpr int oB2 = oW2 + kH * kH;
constexpr int oW3 = oB2 + kH;
constexpr int oB3 = oW3 + kH;
constexpr int kParams = oB3 + 1;
static_assert(kParams == 1313, "parameter layout");

__device__ __forceinline__ float forward_one(float const * P, float const * x, float (&h1)[kH], float (&h2)[kH])
{
#pragma unroll
    for (int k = 0; k < kH; ++k)
    {
        float a = P[oB1 + k];
#pragma unroll
        for (int f = 0; f < kF; ++f)
            a = fmaf(P[oW1 + k * kF + f], x[f], a);
        h1[k] = a > 0.0f ? a : 0.0f;
    }
#pragma unroll 4
    for (int j = 0; j < kH; ++j)
    {
        float a = P[oB2 + j];
#pragma unroll
        for (int k = 0; k < kH; ++k)
            a = fmaf(P[oW2 + j * kH + k], h1[k], a);
        h2[j] = a > 0.0f ? a : 0.0f;
    }
    float y = P[oB3];
#pragma unroll
    for (int j = 0; j < kH; ++j)
        y = fmaf(P[oW3 + j], h2[j], y);
    return y;
}

__global__ void k_mlp_predict(float const * __restrict__ params, float const * __restrict__ X, uint64_t n,
                              float * __restrict__ out)
{
    __shared__ float P[kParams];
    for (int i = threadIdx.x; i < kParams; i += blockDim.x)
        P[i] = params[i];
    __syncthreads();
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
    {
        float x[kF], h1[kH], h2[kH];
#pragma unroll
        for (int f = 0; f < kF; ++f)
            x[f] = X[i * kF + f];
        out[i] = forward_one(P, x, h1, h2);
    }
}

__device__ __forceinline__ float warp_sum(float v)
{
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        v += __shfl_xor_sync(0xFFFFFFFFu, v, o);
    return v;
}

// Gradient of mean((y - log1p(work))^2) over n samples, added into grads; the summed squared error into *sse.
// Each lane handles one sample; the warp sums every parameter's contributions by shuffles, lane 0 adds them to the
// block's shared gradient, and the block adds that to the global one.
__global__ void __launch_bounds__(256) k_mlp_grad(float const * __restrict__ params, float const * __restrict__ X,
                                                  unsigned long long const * __restrict__ work, uint64_t n,
                                                  float scale, float * __restrict__ grads, double * sse)
{
    __shared__ float P[kParams];
    __shared__ float G[kParams];
    for (int i = threadIdx.x; i < kParams; i += blockDim.x)
    {
        P[i] = params[i];
        G[i] = 0.0f;
    }
    __syncthreads();
    int const lane = threadIdx.x & 31;
    uint64_t const warp0 = (blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x) >> 5;
    uint64_t const nwarps = (static_cast<uint64_t>(gridDim.x) * blockDim.x) >> 5;
    double err_acc = 0.0;
    for (uint64_t base = warp0 * 32; base < n; base += nwarps * 32)
    {
        uint64_t const i = base + lane;
        bool const valid = i < n;
        float x[kF], h1[kH], h2[kH];
#pragma unroll
        for (int f = 0; f < kF; ++f)
            x[f] = valid ? X[i * kF + f] : 0.0f;
        float const y = forward_one(P, x, h1, h2);
        float const t = valid ? log1pf(static_cast<float>(work[i])) : y;
        float const e = valid ? y - t : 0.0f;
        err_acc += static_cast<double>(e) * e;
        float const dy = 2.0f * e * scale;
        // output layer
        float s = warp_sum(dy);
        if (lane == 0)
            atomicAdd(&G[oB3], s);
        float dh2[kH];
#pragma unroll
        for (int j = 0; j < kH; ++j)
        {
            s = warp_sum(dy * h2[j]);
            if (lane == 0)
                atomicAdd(&G[oW3 + j], s);
            dh2[j] = h2[j] > 0.0f ? dy * P[oW3 + j] : 0.0f;
        }
        // second hidden layer
        float dh1[kH];
#pragma unroll
        for (int k = 0; k < kH; ++k)
            dh1[k] = 0.0f;
#pragma unroll 2
        for (int j = 0; j < kH; ++j)
        {
            s = warp_sum(dh2[j]);
            if (lane == 0)
                atomicAdd(&G[oB2 + j], s);
#pragma unroll
            for (int k = 0; k < kH; ++k)
            {
                s = warp_sum(dh2[j] * h1[k]);
                if (lane == 0)
                    atomicAdd(&G[oW2 + j * kH + k], s);
                dh1[k] = fmaf(P[oW2 + j * kH + k], dh2[j], dh1[k]);
            }
        }
        // first hidden layer
#pragma unroll 4
        for (int k = 0; k < kH; ++k)
        {
            float const d = h1[k] > 0.0f ? dh1[k] : 0.0f;
            s = warp_sum(d);
            if (lane == 0)
                atomicAdd(&G[oB1 + k], s);
#pragma unroll
            for (int f = 0; f < kF; ++f)
            {
                s = warp_sum(d * x[f]);
                if (lane == 0)
                    atomicAdd(&G[oW1 + k * kF + f], s);
            }
        }
    }
#pragma unroll
    for (int o = 16; o > 0; o >>= 1)
        err_acc += __shfl_xor_sync(0xFFFFFFFFu, err_acc, o);
    if (lane == 0 && err_acc != 0.0)
        atomicAdd(sse, err_acc);
    __syncthreads();
    for (int i = threadIdx.x; i < kParams; i += blockDim.x)
        if (G[i] != 0.0f)
            atomicAdd(&grads[i], G[i]);
}

// Adam (Kingma & Ba, 2015) with bias correction; step counts from 1.
__global__ void k_adam(float * __restrict__ params, float const * __restrict__ grads, float * __restrict__ m,
                       float * __restrict__ v, float lr, float b1, float b2, float eps, float c1, float c2)
{
    int const i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= kParams)
        return;
    float const g = grads[i];
    float const mi = b1 * m[i] + (1.0f - b1) * g;
    float const vi = b2 * v[i] + (1.0f - b2) * g * g;
    m[i] = mi;
    v[i] = vi;
    params[i] -= lr * (mi / c1) / (sqrtf(vi / c2) + eps);
}

__global__ void k_iota(uint32_t * out, uint64_t n)
{
    for (uint64_t i = blockIdx.x * static_cast<uint64_t>(blockDim.x) + threadIdx.x; i < n;
         i += static_cast<uint64_t>(gridDim.x) * blockDim.x)
        out[i] = static_cast<uint32_t>(i);
}

unsigned grid_of(uint64_t n, unsigned block, unsigned per_sm)
{
    uint64_t const want = (n + block - 1) / block;
    return static_cast<unsigned>(
        std::max<uint64_t>(1, std::min<uint64_t>(want, static_cast<uint64_t>(sm_count()) * per_sm)));
}

} // namespace
} // namespace hibf_gb300

using namespace hibf_gb300;

struct hibf_gpu_cost_model
{
    dbuf params, grads, m, v, sse, pred, keys_out, idx, sort_tmp;
    cudaStream_t stream{};
    uint64_t adam_steps{};
};

namespace
{

void sort_desc(hibf_gpu_cost_model * c, float const * d_keys, uint64_t n, uint32_t * d_order, cudaStream_t s)
{
    if (n > 0xFFFFFFFFull)
        fail(HIBF_GPU_ERR_INVALID_ARG, "at most 2^32 - 1 queries");
    c->keys_out.ensure(n * 4);
    c->idx.ensure(n * 4);
    k_iota<<<grid_of(n, 256, 8), 256, 0, s>>>(c->idx.as<uint32_t>(), n);
    HG_CUDA(cudaGetLastError());
    size_t bytes = 0;
    int const items = static_cast<int>(n);
    HG_CUDA(cub::DeviceRadixSort::SortPairsDescending(nullptr, bytes, d_keys, c->keys_out.as<float>(),
                                                      c->idx.as<uint32_t>(), d_order, items, 0, 32, s));
    c->sort_tmp.ensure(std::max<size_t>(bytes, 16));
    HG_CUDA(cub::DeviceRadixSort::SortPairsDescending(c->sort_tmp.p, bytes, d_keys, c->keys_out.as<float>(),
                                                      c->idx.as<uint32_t>(), d_order, items, 0, 32, s));
}

void grad_pass(hibf_gpu_cost_model * c, float const * X, uint64_t const * work, uint64_t n)
{
    HG_CUDA(cudaMemsetAsync(c->grads.p, 0, kParams * 4, c->stream));
    HG_CUDA(cudaMemsetAsync(c->sse.p, 0, 8, c->stream));
    if (!n)
        return;
    k_mlp_grad<<<grid_of((n + 31) / 32 * 32, 256, 4), 256, 0, c->stream>>>(
        c->params.as<float>(), X, reinterpret_cast<unsigned long long const *>(work), n,
        1.0f / static_cast<float>(n), c->grads.as<float>(), c->sse.as<double>());
    HG_CUDA(cudaGetLastError());
}

} // namespace

extern "C"
{

    int hibf_gpu_cost_model_create(uint64_t seed, hibf_gpu_cost_model ** out)
    {
        return guarded(
            [&]
            {
                if (!out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                *out = nullptr;
                require_device();
                auto c = new hibf_gpu_cost_model{};
                try
                {
                    HG_CUDA(cudaStreamCreateWithFlags(&c->stream, cudaStreamNonBlocking));
                    for (dbuf * b : {&c->params, &c->grads, &c->m, &c->v})
                        b->ensure(kParams * 4);
                    c->sse.ensure(8);
                    // He-uniform weights from a seeded splitmix64 stream, zero biases
                    std::vector<float> p(kParams, 0.0f);
                    uint64_t st = seed;
                    auto uni = [&](float bound)
                    { return static_cast<float>((2.0 * hg_unit(hg_next(&st)) - 1.0) * bound); };
                    for (int i = 0; i < kH * kF; ++i)
                        p[oW1 + i] = uni(std::sqrt(6.0f / kF));
                    for (int i = 0; i < kH * kH; ++i)
                        p[oW2 + i] = uni(std::sqrt(6.0f / kH));
                    for (int i = 0; i < kH; ++i)
                        p[oW3 + i] = uni(std::sqrt(6.0f / kH));
                    HG_CUDA(cudaMemcpyAsync(c->params.p, p.data(), kParams * 4, cudaMemcpyHostToDevice, c->stream));
                    HG_CUDA(cudaMemsetAsync(c->m.p, 0, kParams * 4, c->stream));
                    HG_CUDA(cudaMemsetAsync(c->v.p, 0, kParams * 4, c->stream));
                    HG_CUDA(cudaStreamSynchronize(c->stream));
                }
                catch (...)
                {
                    if (c->stream)
                        cudaStreamDestroy(c->stream);
                    delete c;
                    throw;
                }
                *out = c;
            });
    }

    int hibf_gpu_cost_model_destroy(hibf_gpu_cost_model * c)
    {
        if (!c)
            return HIBF_GPU_OK;
        cudaStreamSynchronize(c->stream);
        cudaStreamDestroy(c->stream);
        delete c;
        return HIBF_GPU_OK;
    }

    int hibf_gpu_cost_model_get_params(hibf_gpu_cost_model * c, float * out)
    {
        return guarded(
            [&]
            {
                if (!c || !out)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                HG_CUDA(cudaMemcpyAsync(out, c->params.p, kParams * 4, cudaMemcpyDeviceToHost, c->stream));
                HG_CUDA(cudaStreamSynchronize(c->stream));
            });
    }

    int hibf_gpu_cost_model_set_params(hibf_gpu_cost_model * c, float const * in)
    {
        return guarded(
            [&]
            {
                if (!c || !in)
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                HG_CUDA(cudaMemcpyAsync(c->params.p, in, kParams * 4, cudaMemcpyHostToDevice, c->stream));
                HG_CUDA(cudaMemsetAsync(c->m.p, 0, kParams * 4, c->stream));
                HG_CUDA(cudaMemsetAsync(c->v.p, 0, kParams * 4, c->stream));
                HG_CUDA(cudaStreamSynchronize(c->stream));
                c->adam_steps = 0;
            });
    }

    int hibf_gpu_cost_model_loss_grad_d(hibf_gpu_cost_model * c, float const * d_features, uint64_t const * d_work,
                                        uint64_t n, float * grads, double * loss)
    {
        return guarded(
            [&]
            {
                if (!c || (n && (!d_features || !d_work)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                grad_pass(c, d_features, d_work, n);
                double sse = 0;
                if (grads)
                    HG_CUDA(cudaMemcpyAsync(grads, c->grads.p, kParams * 4, cudaMemcpyDeviceToHost, c->stream));
                HG_CUDA(cudaMemcpyAsync(&sse, c->sse.p, 8, cudaMemcpyDeviceToHost, c->stream));
                HG_CUDA(cudaStreamSynchronize(c->stream));
                if (loss)
                    *loss = n ? sse / static_cast<double>(n) : 0.0;
            });
    }

    int hibf_gpu_cost_model_train_d(hibf_gpu_cost_model * c, float const * d_features, uint64_t const * d_work,
                                    uint64_t n, uint32_t steps, float lr, double * loss)
    {
        return guarded(
            [&]
            {
                if (!c || n == 0 || !d_features || !d_work || !(lr > 0.0f))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "bad argument");
                float const b1 = 0.9f, b2 = 0.999f, eps = 1e-8f;
                for (uint32_t k = 0; k < steps; ++k)
                {
                    grad_pass(c, d_features, d_work, n);
                    ++c->adam_steps;
                    float const c1 = 1.0f - std::pow(b1, static_cast<float>(c->adam_steps));
                    float const c2 = 1.0f - std::pow(b2, static_cast<float>(c->adam_steps));
                    k_adam<<<(kParams + 255) / 256, 256, 0, c->stream>>>(c->params.as<float>(), c->grads.as<float>(),
                                                                        c->m.as<float>(), c->v.as<float>(), lr, b1, b2,
                                                                        eps, c1, c2);
                    HG_CUDA(cudaGetLastError());
                }
                // loss of the final parameters
                grad_pass(c, d_features, d_work, n);
                double sse = 0;
                HG_CUDA(cudaMemcpyAsync(&sse, c->sse.p, 8, cudaMemcpyDeviceToHost, c->stream));
                HG_CUDA(cudaStreamSynchronize(c->stream));
                if (loss)
                    *loss = sse / static_cast<double>(n);
            });
    }

    int hibf_gpu_cost_model_predict_d(hibf_gpu_cost_model * c, float const * d_features, uint64_t n, float * d_pred,
                                      void * stream)
    {
        return guarded(
            [&]
            {
                if (!c || (n && (!d_features || !d_pred)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (!n)
                    return;
                cudaStream_t const s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
                k_mlp_predict<<<grid_of(n, 256, 8), 256, 0, s>>>(c->params.as<float>(), d_features, n, d_pred);
                HG_CUDA(cudaGetLastError());
            });
    }

    int hibf_gpu_sort_desc_d(hibf_gpu_cost_model * c, float const * d_keys, uint64_t n, uint32_t * d_order,
                             void * stream)
    {
        return guarded(
            [&]
            {
                if (!c || (n && (!d_keys || !d_order)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (!n)
                    return;
                sort_desc(c, d_keys, n, d_order, stream ? static_cast<cudaStream_t>(stream) : c->stream);
            });
    }

    int hibf_gpu_cost_model_order_d(hibf_gpu_cost_model * c, float const * d_features, uint64_t n, uint32_t * d_order,
                                    void * stream)
    {
        return guarded(
            [&]
            {
                if (!c || (n && (!d_features || !d_order)))
                    fail(HIBF_GPU_ERR_INVALID_ARG, "null argument");
                if (!n)
                    return;
                cudaStream_t const s = stream ? static_cast<cudaStream_t>(stream) : c->stream;
                c->pred.ensure(n * 4);
                k_mlp_predict<<<grid_of(n, 256, 8), 256, 0, s>>>(c->params.as<float>(), d_features, n,
                                                               c->pred.as<float>());
                HG_CUDA(cudaGetLastError());
                sort_desc(c, c->pred.as<float>(), n, d_order, s);
            });
    }

} // extern "C"
