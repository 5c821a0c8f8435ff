// The graph nodes either side of the path tracer that run on the GPU: Accumulate (progressive
// mean over frames) and the error metrics of Error Plot.
//
// Accumulate restates accumulate.slang:233-257 for a static camera: the history of a pixel is
// its own previous output (no motion-vector reprojection or GBuffer validation, which a static
// camera never rejects) and the firefly filter is off (its default). Error Plot restates
// error_to_buffer.slang: per-texel (reference - input)^2 or |reference - input| summed per
// channel, here reduced on the device in a fixed order.
#include "context.h"
#include "device_math.cuh"

#include <cmath>
#include <vector>

namespace gbpt {
namespace {

GBPT_DI bool finite4(float4 v) {
    return isfinite(v.x) && isfinite(v.y) && isfinite(v.z) && isfinite(v.w);
}

// lerp(prev, src, a) = prev + a * (src - prev), with the operations rounded one at a time
GBPT_DI float lerp_rn(float x, float y, float a) { return __fadd_rn(x, __fmul_rn(a, __fsub_rn(y, x))); }

__global__ void k_accumulate(const float4* __restrict__ src, float4* out, float* history,
                             uint64_t n, float accum_alpha, float max_history, int clear) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const float4 s = src[i];
        const float4 prev = out[i];
        const float prev_hist = history[i];
        if (!clear && prev_hist > 0.f && finite4(prev)) {
            const float nh = fminf(prev_hist + 1.0f, max_history);
            const float a = fmaxf(1.0f - accum_alpha, __fdiv_rn(1.0f, nh));
            out[i] = make_float4(lerp_rn(prev.x, s.x, a), lerp_rn(prev.y, s.y, a),
                                 lerp_rn(prev.z, s.z, a), lerp_rn(prev.w, s.w, a));
            history[i] = nh;
        } else {
            out[i] = s;
            history[i] = 1.0f;
        }
    }
}

constexpr int kErrBlocks = 1024;

// Per-block partial sums of (ref - in)^2 and |ref - in| per channel, in double, in a fixed order
// (block-strided texels, then a fixed shuffle tree and a fixed sum over warps).
__global__ void __launch_bounds__(256) k_error_partial(const float4* __restrict__ ref,
                                                       const float4* __restrict__ in, uint64_t n,
                                                       double* partial) {
    double acc[8] = {0, 0, 0, 0, 0, 0, 0, 0};
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x) {
        const float4 a = ref[i], b = in[i];
        const double d[4] = {(double)a.x - b.x, (double)a.y - b.y, (double)a.z - b.z,
                             (double)a.w - b.w};
        for (int c = 0; c < 4; ++c) {
            acc[c] += d[c] * d[c];
            acc[4 + c] += fabs(d[c]);
        }
    }
    __shared__ double warp_sums[8][8];
    const int lane = threadIdx.x & 31, warp = threadIdx.x >> 5;
    for (int c = 0; c < 8; ++c) {
        double v = acc[c];
        for (int off = 16; off > 0; off >>= 1) v += __shfl_xor_sync(0xFFFFFFFFu, v, off);
        if (lane == 0) warp_sums[warp][c] = v;
    }
    __syncthreads();
    if (threadIdx.x < 8) {
        double s = 0;
        for (int w = 0; w < 8; ++w) s += warp_sums[w][threadIdx.x];
        partial[blockIdx.x * 8 + threadIdx.x] = s;
    }
}

// The GBuffer node's "emission" image: RGBA32F texels (alpha 1) from the GBuffer texels.
__global__ void k_gbuffer_emission(const gbpt_gbuffer_texel* __restrict__ g, float4* out,
                                   uint64_t n) {
    for (uint64_t i = blockIdx.x * (uint64_t)blockDim.x + threadIdx.x; i < n;
         i += (uint64_t)gridDim.x * blockDim.x)
        out[i] = make_float4(g[i].emission[0], g[i].emission[1], g[i].emission[2], 1.0f);
}

} // namespace

int gbuffer_emission(gbpt_ctx* ctx, const gbpt_gbuffer_texel* texels, float* out_device,
                     uint64_t n) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (n == 0) return GBPT_OK;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int grid = (int)std::min<uint64_t>((n + 255) / 256, (uint64_t)num_sms() * 16);
    k_gbuffer_emission<<<grid, 256, 0, ctx->stream>>>(texels, (float4*)out_device, n);
    GBPT_CUDA_CHECK(cudaGetLastError());
    return GBPT_OK;
}

} // namespace gbpt

using namespace gbpt;

extern "C" {

GBPT_API int gbpt_accumulate(gbpt_ctx* ctx, const float* src_device, float* out_device,
                             float* history_device, uint64_t texels, float alpha,
                             float max_history, int clear) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (texels && (!src_device || !out_device || !history_device)) {
        set_error("gbpt_accumulate: null buffer");
        return GBPT_ERR_INVALID;
    }
    if (!(alpha >= 0.f && alpha <= 1.f) || !(max_history >= 1.f)) {
        set_error("gbpt_accumulate: alpha must be in [0, 1] and max history at least 1");
        return GBPT_ERR_INVALID;
    }
    if (texels == 0) return GBPT_OK;
    std::lock_guard<std::mutex> lk(ctx->mu);
    const int grid = (int)std::min<uint64_t>((texels + 255) / 256, (uint64_t)num_sms() * 16);
    k_accumulate<<<grid, 256, 0, ctx->stream>>>((const float4*)src_device, (float4*)out_device,
                                                history_device, texels, alpha, max_history,
                                                clear);
    GBPT_CUDA_CHECK(cudaGetLastError());
    return GBPT_OK;
}

GBPT_API int gbpt_error_metrics(gbpt_ctx* ctx, const float* reference_device,
                                const float* input_device, uint64_t texels, double* out8) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!out8 || (texels && (!reference_device || !input_device))) {
        set_error("gbpt_error_metrics: null pointer");
        return GBPT_ERR_INVALID;
    }
    for (int c = 0; c < 8; ++c) out8[c] = 0.0;
    if (texels == 0) return GBPT_OK;
    std::lock_guard<std::mutex> lk(ctx->mu);
    double* partial = nullptr;
    GBPT_CUDA_CHECK(cudaMallocAsync((void**)&partial, kErrBlocks * 8 * sizeof(double), ctx->stream));
    k_error_partial<<<kErrBlocks, 256, 0, ctx->stream>>>((const float4*)reference_device,
                                                         (const float4*)input_device, texels,
                                                         partial);
    std::vector<double> h(kErrBlocks * 8);
    const cudaError_t e1 = cudaMemcpyAsync(h.data(), partial, h.size() * sizeof(double),
                                           cudaMemcpyDeviceToHost, ctx->stream);
    cudaFreeAsync(partial, ctx->stream);
    GBPT_CUDA_CHECK(e1);
    GBPT_CUDA_CHECK(cudaStreamSynchronize(ctx->stream));
    for (int b = 0; b < kErrBlocks; ++b)
        for (int c = 0; c < 8; ++c) out8[c] += h[b * 8 + c];
    for (int c = 0; c < 8; ++c) out8[c] /= (double)texels;
    return GBPT_OK;
}

} // extern "C"
