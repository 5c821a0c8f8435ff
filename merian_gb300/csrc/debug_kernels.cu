// Test hooks: the device BSDF code run in isolation, so tests can compare it sample by sample with
// the CPU oracle and run merian's BSDF property checks (tests/bsdf/bsdf-checks.slang) on the GPU.
#include "device_math.cuh"
#include "host_common.h"

#include <cuda_runtime.h>

namespace gbpt {
namespace {

__global__ void k_material_samples(float4 m0, float4 m1, float4 m2, float4 m3, int front, float ior,
                                   float3 wi, uint32_t seed, uint32_t n, float* out) {
    const uint32_t i = blockIdx.x * blockDim.x + threadIdx.x;
    if (i >= n) return;
    const Material m = material_from_record(m0, m1, m2, m3, front != 0, ior);
    Pcg rng{pcg4d16(i, seed, 0u, 0u)};
    const BsdfSample s = material_sample(m, wi, rng);
    float* o = out + 12ull * i;
    o[0] = s.wo.x;
    o[1] = s.wo.y;
    o[2] = s.wo.z;
    o[3] = s.pdf;
    o[4] = s.weight.x;
    o[5] = s.weight.y;
    o[6] = s.weight.z;
    o[7] = s.valid ? 1.f : 0.f;
    const float3 e = s.valid ? material_eval(m, wi, s.wo) : f3(0.f, 0.f, 0.f);
    o[8] = e.x;
    o[9] = e.y;
    o[10] = e.z;
    o[11] = s.valid ? material_pdf(m, wi, s.wo) : 0.f;
}

struct CheckBsdf {
    int kind;
    float3 albedo, f0;
    float alpha, alpha_y, ior_f0, eta;
    template <class G> GBPT_DI BsdfSample sample(float3 wi, G& rng) const {
        switch (kind) {
        case 0: return lambert_sample(albedo, wi, rng);
        case 1: return ggx_sample(alpha, alpha_y, wi, rng);
        case 2: return conductor_sample(alpha, alpha, f0, wi, rng);
        case 3: return rough_dielectric_sample(alpha, eta, albedo, wi, rng);
        default: {
            Material m;
            m.model = 1u;
            m.base = albedo;
            m.ax = m.ay = alpha;
            m.f0 = ior_f0;
            return opaque_sample(m, wi, rng);
        }
        }
    }
    GBPT_DI float3 eval(float3 wi, float3 wo) const {
        switch (kind) {
        case 0: return lambert_eval(albedo, wi, wo);
        case 1: {
            const float g = ggx_eval(alpha, alpha_y, wi, wo);
            return f3(g, g, g);
        }
        case 2: return conductor_eval(alpha, alpha, f0, wi, wo);
        case 3: return rough_dielectric_eval(alpha, eta, albedo, wi, wo);
        default: {
            Material m;
            m.model = 1u;
            m.base = albedo;
            m.ax = m.ay = alpha;
            m.f0 = ior_f0;
            return opaque_eval(m, wi, wo);
        }
        }
    }
    GBPT_DI float pdf(float3 wi, float3 wo) const {
        switch (kind) {
        case 0: return lambert_pdf(wi, wo);
        case 1: return ggx_pdf(alpha, alpha_y, wi, wo);
        case 2: return ggx_pdf(alpha, alpha, wi, wo);
        case 3: return rough_dielectric_pdf(alpha, eta, wi, wo);
        default: {
            Material m;
            m.model = 1u;
            m.base = albedo;
            m.ax = m.ay = alpha;
            m.f0 = ior_f0;
            return opaque_pdf(m, wi, wo);
        }
        }
    }
};

GBPT_DI float acc_err(float acc, float v) { return isfinite(v) ? fmaxf(acc, v) : 1e30f; }

// One thread, as the reference check (bsdf-checks.slang:30): Welford means, then a 256 x 512
// midpoint quadrature of the hemisphere.
__global__ void k_bsdf_check(CheckBsdf b, float3 wi, uint32_t n, uint32_t seed, float* out) {
    if (blockIdx.x != 0 || threadIdx.x != 0) return;
    XorShift rng{seed | 1u};
    float3 mean_w = f3(0.f, 0.f, 0.f), m2_w = f3(0.f, 0.f, 0.f);
    float mean_cos = 0.f, m2_cos = 0.f, max_w_err = 0.f, max_pdf_err = 0.f;
    uint32_t valid = 0;
    for (uint32_t i = 0; i < n; ++i) {
        float3 w = f3(0.f, 0.f, 0.f);
        float c = 0.f;
        const BsdfSample s = b.sample(wi, rng);
        if (s.valid) {
            valid++;
            w = s.weight;
            c = s.wo.z / s.pdf;
            const float pref = b.pdf(wi, s.wo);
            const float3 eref = b.eval(wi, s.wo);
            max_pdf_err = acc_err(max_pdf_err, fabsf(s.pdf - pref) /
                                                   (fmaxf(fabsf(s.pdf), fabsf(pref)) + 1e-6f));
            if (pref > 0.f) max_w_err = acc_err(max_w_err, length(s.weight - eref / pref));
        }
        const float inv_i = 1.0f / (float)(i + 1);
        const float3 dw = w - mean_w;
        mean_w = mean_w + dw * inv_i;
        m2_w = m2_w + dw * (w - mean_w);
        const float dc = c - mean_cos;
        mean_cos += dc * inv_i;
        m2_cos += dc * (c - mean_cos);
    }
    const float inv_n = 1.0f / (float)n;
    const uint32_t NT = 256, NP = 512;
    const float dth = (kPi * 0.5f) / (float)NT, dph = kTwoPi / (float)NP;
    float pdf_int = 0.f, max_recip = 0.f;
    for (uint32_t ti = 0; ti < NT; ++ti) {
        const float th = ((float)ti + 0.5f) * dth;
        const float ct = cosf(th), st = sinf(th);
        for (uint32_t pi = 0; pi < NP; ++pi) {
            const float ph = ((float)pi + 0.5f) * dph;
            const float3 wo = f3(st * cosf(ph), st * sinf(ph), ct);
            pdf_int += b.pdf(wi, wo) * st * dth * dph;
            const float3 fio = b.eval(wi, wo) / wo.z;
            const float3 foi = b.eval(wo, wi) / wi.z;
            const float3 d = f3(fabsf(fio.x - foi.x), fabsf(fio.y - foi.y), fabsf(fio.z - foi.z));
            const float3 m = f3(fmaxf(fabsf(fio.x), fabsf(foi.x)) + 1e-6f,
                                fmaxf(fabsf(fio.y), fabsf(foi.y)) + 1e-6f,
                                fmaxf(fabsf(fio.z), fabsf(foi.z)) + 1e-6f);
            max_recip = acc_err(max_recip, fmaxf(fmaxf(d.x / m.x, d.y / m.y), d.z / m.z));
        }
    }
    out[0] = mean_w.x;
    out[1] = mean_w.y;
    out[2] = mean_w.z;
    out[3] = sqrtf(m2_w.x) * inv_n;
    out[4] = sqrtf(m2_w.y) * inv_n;
    out[5] = sqrtf(m2_w.z) * inv_n;
    out[6] = mean_cos;
    out[7] = sqrtf(m2_cos) * inv_n;
    out[8] = (float)valid;
    out[9] = max_w_err;
    out[10] = max_pdf_err;
    out[11] = pdf_int;
    out[12] = max_recip;
    out[13] = out[14] = out[15] = 0.f;
}

int finish(float* d_out, float* host, size_t bytes, const char* what) {
    cudaError_t e = cudaGetLastError();
    if (e == cudaSuccess) e = cudaMemcpy(host, d_out, bytes, cudaMemcpyDeviceToHost);
    cudaFree(d_out);
    if (e != cudaSuccess) {
        set_error(std::string(what) + ": " + cudaGetErrorString(e));
        return GBPT_ERR_CUDA;
    }
    return GBPT_OK;
}

} // namespace
} // namespace gbpt

using namespace gbpt;

extern "C" GBPT_API int gbpt_debug_material_samples(const gbpt_material* material,
                                                    int front_facing, float ior, const float wi[3],
                                                    uint32_t seed, uint32_t n, float* out_host) {
    if (!material || !wi || !out_host || n == 0 || n > (1u << 24) ||
        material->model > GBPT_MATERIAL_OPENPBR_TRANSMISSION) {
        set_error("gbpt_debug_material_samples: invalid arguments");
        return GBPT_ERR_INVALID;
    }
    float4 rec[5];
    std::memcpy(rec, material, sizeof(rec));
    float* d = nullptr;
    const size_t bytes = (size_t)n * 12 * sizeof(float);
    if (cudaMalloc((void**)&d, bytes) != cudaSuccess) {
        set_error("gbpt_debug_material_samples: cudaMalloc failed");
        return GBPT_ERR_NO_MEMORY;
    }
    k_material_samples<<<(n + 127) / 128, 128>>>(rec[0], rec[1], rec[2], rec[3], front_facing, ior,
                                                  make_float3(wi[0], wi[1], wi[2]), seed, n, d);
    return finish(d, out_host, bytes, "gbpt_debug_material_samples");
}

extern "C" GBPT_API int gbpt_debug_bsdf_check(int kind, const float wi[3], const float albedo[3],
                                              float alpha, float alpha_y, const float f0[3],
                                              float ior_f0, float eta, uint32_t n_samples,
                                              uint32_t seed, float* out16) {
    if (!wi || !albedo || !f0 || !out16 || kind < 0 || kind > 4 || n_samples == 0) {
        set_error("gbpt_debug_bsdf_check: invalid arguments");
        return GBPT_ERR_INVALID;
    }
    CheckBsdf b;
    b.kind = kind;
    b.albedo = make_float3(albedo[0], albedo[1], albedo[2]);
    b.f0 = make_float3(f0[0], f0[1], f0[2]);
    b.alpha = alpha;
    b.alpha_y = alpha_y;
    b.ior_f0 = ior_f0;
    b.eta = eta;
    float* d = nullptr;
    if (cudaMalloc((void**)&d, 16 * sizeof(float)) != cudaSuccess) {
        set_error("gbpt_debug_bsdf_check: cudaMalloc failed");
        return GBPT_ERR_NO_MEMORY;
    }
    k_bsdf_check<<<1, 1>>>(b, make_float3(wi[0], wi[1], wi[2]), n_samples, seed, d);
    return finish(d, out16, 16 * sizeof(float), "gbpt_debug_bsdf_check");
}
