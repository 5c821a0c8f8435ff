// The context object behind the C ABI and the helpers its translation units share (api.cpp,
// server.cpp). Host-only C++.
#pragma once

#include "gbpt.h"
#include "runtime.h"

#include <array>
#include <cstdint>
#include <map>
#include <memory>
#include <mutex>
#include <string>

#include <cuda_runtime.h>

namespace gbpt {
void set_error(const std::string& msg);
struct Server; // server.cpp
struct ServerDeleter {
    void operator()(Server* s) const;
};
using ServerPtr = std::unique_ptr<Server, ServerDeleter>;
// Stops the server thread (cancelling queued requests) and frees its resources.
void server_shutdown(ServerPtr& s);
} // namespace gbpt

struct gbpt_ctx {
    int device = 0;
    cudaStream_t stream = nullptr;
    bool own_stream = false;
    std::mutex mu;
    std::map<uint32_t, gbpt::SceneGPU> scenes; // node addresses stay valid until erased
    std::map<uint32_t, int> scene_users;       // server requests holding a scene (queued or running)
    uint32_t next_scene = 1;
    gbpt::Work work;
    gbpt::TickEngine batch; // gbpt_render_batch, over `work`
    // gbpt_tuning.streams = 2: the second tick stream, its work buffers, and the events that
    // order it after and before the context stream
    gbpt::Work work2;
    gbpt::TickEngine batch2; // gbpt_render_batch's odd ticks, over `work2`
    cudaStream_t stream2 = nullptr;
    cudaEvent_t ev_fork = nullptr, ev_join = nullptr;
    // schedule of gbpt_render* and gbpt_render_batch: paths per tick (0 = default), material sort
    // override (-1 = as each request asks), CUDA graphs
    gbpt_tuning tuning{0, -1, 0, GBPT_BVH_SPLIT, 0, 0, 0, 0};
    // gbpt_autotune's results by (log2 triangles, log2 paths, path length, NEE, roulette depth)
    struct TuneResult {
        gbpt_tuning tuning;
        std::array<double, GBPT_AUTOTUNE_CANDIDATES> ms;
    };
    std::map<std::array<int, 5>, TuneResult> tune_cache;
    unsigned long long* d_misc = nullptr; // [0] nodes, [1] tris, [2] error word, [4..7] SIMT steps
    gbpt_hit* d_hits = nullptr;
    uint64_t hits_cap = 0;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    gbpt::Profile prof;
    gbpt::ServerPtr server;
};

namespace gbpt {

#define GBPT_CUDA_CHECK(call)                                                                      \
    do {                                                                                           \
        const cudaError_t e_ = (call);                                                             \
        if (e_ != cudaSuccess) {                                                                   \
            ::gbpt::set_error(std::string(#call) + ": " + cudaGetErrorString(e_));                 \
            return e_ == cudaErrorMemoryAllocation ? GBPT_ERR_NO_MEMORY : GBPT_ERR_CUDA;           \
        }                                                                                          \
    } while (0)

// The traversal schedule a tuning asks for (0 fields: the defaults).
TraceSched sched_of(const gbpt_tuning& t);
// Null check and cudaSetDevice for the context's device.
int check_ctx(gbpt_ctx* ctx);
// Camera / parameter validation shared by every render entry point.
int validate_params(const gbpt_camera* cam, const gbpt_render_params* p);
// Seconds on the host's steady clock (request timestamps).
double host_clock();
// The GBuffer node's emission image: n RGBA32F texels (alpha 1) from n GBuffer texels, device
// memory, enqueued on the context stream (nodes.cu).
int gbuffer_emission(gbpt_ctx* ctx, const gbpt_gbuffer_texel* texels, float* out_device,
                     uint64_t n);

} // namespace gbpt
