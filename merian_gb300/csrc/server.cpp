// The request server: continuous batching of render requests over the tick engine.
//
// merian renders one request per graph iteration on the calling thread (Graph::run_node ->
// RenderPT::process, graph.cpp:323-360). The server instead keeps scenes resident and runs one
// host thread that, tick after tick,
//   1. admits queued requests in arrival order while their outputs fit the output arena (device
//      memory reserved from free HBM when the server starts): admission by free HBM;
//   2. plans the next tick over the admitted requests (oldest first, whole pixels, up to the wave
//      size and 256 requests) and enqueues it on the server's stream, one tick ahead of the GPU;
//   3. when a tick has run, completes the requests whose last pixels it held: host outputs are
//      copied out, arena space is freed and waiters are woken.
// A request that arrives while others run joins the next tick, so its work overlaps theirs on
// the device. Every pixel is rendered within one tick from its own (pixel, frame, sample) seeds
// and summed in a fixed order, so a result is bit-identical alone and in any mix.
#include "context.h"
#include "gbpt.h"
#include "runtime.h"

#include <algorithm>
#include <condition_variable>
#include <cstring>
#include <deque>
#include <map>
#include <memory>
#include <mutex>
#include <string>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

namespace gbpt {

namespace {

constexpr uint64_t kArenaAlign = 256;
constexpr int kTicksAhead = 2; // ticks enqueued before the host waits for the oldest

uint64_t align_up(uint64_t x) { return (x + kArenaAlign - 1) & ~(kArenaAlign - 1); }

// First-fit allocator over [0, size) with coalescing free blocks.
class ArenaAlloc {
  public:
    void reset(uint64_t size) {
        free_.clear();
        if (size) free_[0] = size;
    }
    bool alloc(uint64_t bytes, uint64_t& off) {
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second < bytes) continue;
            off = it->first;
            const uint64_t rest = it->second - bytes;
            free_.erase(it);
            if (rest) free_[off + bytes] = rest;
            return true;
        }
        return false;
    }
    void release(uint64_t off, uint64_t bytes) {
        if (!bytes) return;
        auto it = free_.emplace(off, bytes).first;
        auto next = std::next(it);
        if (next != free_.end() && it->first + it->second == next->first) {
            it->second += next->second;
            free_.erase(next);
        }
        if (it != free_.begin()) {
            auto prev = std::prev(it);
            if (prev->first + prev->second == it->first) {
                prev->second += it->second;
                free_.erase(it);
            }
        }
    }

  private:
    std::map<uint64_t, uint64_t> free_;
};

} // namespace

struct ServerReq {
    uint64_t ticket = 0;
    gbpt_request req{};
    std::vector<uint32_t> pixels; // copy of the caller's list
    const SceneGPU* scene = nullptr;
    uint32_t n_pix = 0;
    int state = GBPT_REQ_QUEUED;
    int error = GBPT_OK;
    bool cancel = false;
    double t_submit = 0, t_admit = 0, t_done = 0;
    uint64_t arena_off = 0, arena_bytes = 0;
    float4* d_out = nullptr;
    TickItem item;
    uint64_t last_tick = 0; // sequence number of the last tick holding its pixels
    bool uploaded = false;
};

struct Server {
    gbpt_ctx* ctx = nullptr;
    gbpt_server_config cfg{};
    cudaStream_t stream = nullptr, copy_stream = nullptr;
    Work work;
    TickEngine engine;
    int sort_override = -1; // the context tuning's material-sort override at start
    unsigned char* arena = nullptr;
    uint64_t arena_bytes = 0;
    ArenaAlloc alloc;
    uint32_t* h_flags = nullptr; // pinned, one error word per tick slot
    std::vector<cudaEvent_t> events;

    std::mutex mu;
    std::condition_variable wake; // server thread: submissions, cancels, stop
    std::condition_variable done; // waiters
    std::deque<std::shared_ptr<ServerReq>> queued;
    std::vector<std::shared_ptr<ServerReq>> active; // admitted, oldest first
    std::unordered_map<uint64_t, std::shared_ptr<ServerReq>> all;
    uint64_t next_ticket = 1;
    bool stop = false;
    std::thread thread;
    // totals
    uint64_t ticks = 0, launches = 0, paths = 0, completed = 0;
    std::string fatal; // first CUDA failure of the server thread

    struct InFlight {
        uint64_t seq;
        cudaEvent_t ev;
        int slot;
        std::vector<std::shared_ptr<ServerReq>> members;
    };
    std::deque<InFlight> inflight;

    void run();
    bool admit_locked(std::vector<std::shared_ptr<ServerReq>>& admitted);
    void finish(const std::shared_ptr<ServerReq>& r, int state, int error);
    void release_scene(const ServerReq& r);
    void fail_all(int error, const std::string& why);
};

void Server::release_scene(const ServerReq& r) {
    std::lock_guard<std::mutex> lk(ctx->mu);
    auto it = ctx->scene_users.find(r.req.scene);
    if (it != ctx->scene_users.end() && --it->second <= 0) ctx->scene_users.erase(it);
}

// Called on the server thread without `mu` held.
void Server::finish(const std::shared_ptr<ServerReq>& r, int state, int error) {
    release_scene(*r);
    std::lock_guard<std::mutex> lk(mu);
    alloc.release(r->arena_off, r->arena_bytes);
    r->arena_bytes = 0;
    r->state = state;
    r->error = error;
    r->t_done = host_clock();
    active.erase(std::remove(active.begin(), active.end(), r), active.end());
    ++completed;
    done.notify_all();
}

bool Server::admit_locked(std::vector<std::shared_ptr<ServerReq>>& admitted) {
    const uint32_t max_active = cfg.max_active ? cfg.max_active : 1024u;
    bool any = false;
    while (!queued.empty() && active.size() < max_active) {
        std::shared_ptr<ServerReq> r = queued.front();
        const uint64_t need = (r->req.out_host ? align_up((uint64_t)r->n_pix * 16) : 0) +
                              align_up((uint64_t)r->pixels.size() * 4);
        uint64_t off = 0;
        if (need && !alloc.alloc(need, off)) break; // oldest first: wait for space
        queued.pop_front();
        r->arena_off = off;
        r->arena_bytes = need;
        r->state = GBPT_REQ_RUNNING;
        r->t_admit = host_clock();
        active.push_back(r);
        admitted.push_back(r);
        any = true;
    }
    return any;
}

void Server::fail_all(int error, const std::string& why) {
    std::vector<std::shared_ptr<ServerReq>> victims;
    {
        std::lock_guard<std::mutex> lk(mu);
        if (fatal.empty()) fatal = why;
        victims = active;
        for (auto& q : queued) victims.push_back(q);
        queued.clear();
    }
    for (auto& r : victims) finish(r, GBPT_REQ_FAILED, error);
}

void Server::run() {
    cudaSetDevice(ctx->device);
    uint64_t seq = 0, completed_seq = 0;
    std::vector<std::shared_ptr<ServerReq>> admitted;
    std::vector<TickItem*> items;
    std::vector<std::shared_ptr<ServerReq>> sched;
    while (true) {
        admitted.clear();
        bool have_work = false;
        {
            std::unique_lock<std::mutex> lk(mu);
            while (true) {
                admit_locked(admitted);
                // cancelled requests stop taking ticks; they finish once their ticks have run
                for (auto& r : active)
                    if (r->cancel) r->item.cursor = r->item.pixel_count;
                have_work = false;
                for (auto& r : active)
                    if (r->item.cursor < r->item.pixel_count) have_work = true;
                const bool finishing = std::any_of(active.begin(), active.end(), [&](auto& r) {
                    return r->item.cursor >= r->item.pixel_count && r->last_tick <= completed_seq;
                });
                if (have_work || !inflight.empty() || finishing || !admitted.empty()) break;
                if (stop && queued.empty() && active.empty()) return;
                wake.wait(lk);
            }
            sched = active;
        }
        // pixel lists of newly admitted requests, and their device outputs
        for (auto& r : admitted) {
            unsigned char* base = arena + r->arena_off;
            uint64_t at = 0;
            r->item.scene = r->scene;
            r->item.camera = r->req.camera;
            r->item.params = r->req.params;
            if (sort_override >= 0) r->item.params.sort_materials = sort_override;
            r->item.pixel_count = r->n_pix;
            if (r->req.out_host) {
                r->d_out = (float4*)base;
                at += align_up((uint64_t)r->n_pix * 16);
            } else {
                r->d_out = (float4*)r->req.out_device;
            }
            r->item.out_device = r->d_out;
            r->item.pixels_device = nullptr;
            if (!r->pixels.empty()) {
                uint32_t* d_list = (uint32_t*)(base + at);
                if (cudaMemcpyAsync(d_list, r->pixels.data(), r->pixels.size() * 4,
                                    cudaMemcpyHostToDevice, stream) != cudaSuccess) {
                    fail_all(GBPT_ERR_CUDA, "pixel list upload failed");
                    continue;
                }
                r->item.pixels_device = d_list;
            }
            if (r->req.params.spp == 0) r->item.cursor = r->item.pixel_count; // zeros, no tick
            r->uploaded = true;
        }
        // enqueue the next tick while fewer than kTicksAhead are in flight
        if (have_work && (int)inflight.size() < kTicksAhead) {
            items.clear();
            std::vector<uint32_t> before;
            for (auto& r : sched) {
                if (!r->uploaded || r->item.cursor >= r->item.pixel_count) continue;
                items.push_back(&r->item);
            }
            before.reserve(items.size());
            for (TickItem* it : items) before.push_back(it->cursor);
            uint64_t n_paths = 0, nl = 0;
            const int slot = (int)(seq % kTicksAhead);
            const int rc = tick_enqueue(engine, items.data(), (uint32_t)items.size(), &n_paths,
                                        nullptr, &nl, nullptr, nullptr);
            if (rc != GBPT_OK) {
                fail_all(rc, "tick enqueue failed: " + cuda_error_string(cudaGetLastError()));
                continue;
            }
            if (n_paths > 0) {
                ++seq;
                InFlight f;
                f.seq = seq;
                f.slot = slot;
                f.ev = events[slot];
                for (auto& r : sched) {
                    if (!r->uploaded) continue;
                    for (size_t k = 0; k < items.size(); ++k)
                        if (items[k] == &r->item && items[k]->cursor != before[k]) {
                            r->last_tick = seq;
                            f.members.push_back(r);
                        }
                }
                cudaMemcpyAsync(h_flags + slot, work.counters + 3, 4, cudaMemcpyDeviceToHost,
                                stream);
                cudaMemsetAsync(work.counters + 3, 0, 4, stream);
                cudaEventRecord(f.ev, stream);
                inflight.push_back(std::move(f));
                std::lock_guard<std::mutex> lk(mu);
                ++ticks;
                launches += nl;
                paths += n_paths;
            }
        }
        // retire the oldest tick when the pipeline is full or nothing more can be enqueued
        const bool more = std::any_of(sched.begin(), sched.end(), [](auto& r) {
            return r->uploaded && r->item.cursor < r->item.pixel_count;
        });
        if (!inflight.empty() && ((int)inflight.size() >= kTicksAhead || !more)) {
            InFlight f = std::move(inflight.front());
            inflight.pop_front();
            if (cudaEventSynchronize(f.ev) != cudaSuccess) {
                fail_all(GBPT_ERR_CUDA, "tick failed: " + cuda_error_string(cudaGetLastError()));
                inflight.clear();
                continue;
            }
            completed_seq = f.seq;
            if (h_flags[f.slot]) {
                for (auto& r : f.members) r->error = GBPT_ERR_DEVICE;
                h_flags[f.slot] = 0;
            }
        }
        // complete the requests whose ticks have all run
        for (auto& r : sched) {
            if (!r->uploaded || r->item.cursor < r->item.pixel_count || r->last_tick > completed_seq)
                continue;
            if (r->state != GBPT_REQ_RUNNING) continue;
            int state = GBPT_REQ_DONE, err = r->error;
            if (r->cancel) state = GBPT_REQ_CANCELLED;
            else if (err != GBPT_OK) state = GBPT_REQ_FAILED;
            else if (r->req.params.spp == 0) {
                // no samples: the output is zero (gbpt_render's convention)
                const size_t bytes = (size_t)r->n_pix * sizeof(float4);
                if (r->req.out_host) std::memset(r->req.out_host, 0, bytes);
                else if (cudaMemsetAsync(r->req.out_device, 0, bytes, copy_stream) != cudaSuccess ||
                         cudaStreamSynchronize(copy_stream) != cudaSuccess) {
                    state = GBPT_REQ_FAILED;
                    err = GBPT_ERR_CUDA;
                }
            } else if (r->req.out_host) {
                const cudaError_t e =
                    cudaMemcpyAsync(r->req.out_host, r->d_out, (size_t)r->n_pix * sizeof(float4),
                                    cudaMemcpyDeviceToHost, copy_stream);
                if (e != cudaSuccess || cudaStreamSynchronize(copy_stream) != cudaSuccess) {
                    state = GBPT_REQ_FAILED;
                    err = GBPT_ERR_CUDA;
                }
            }
            finish(r, state, err);
        }
    }
}

void ServerDeleter::operator()(Server* s) const { delete s; }

void server_shutdown(ServerPtr& s) {
    if (!s) return;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        s->stop = true;
        // queued requests are cancelled; admitted ones run to completion
        for (auto& r : s->queued) {
            r->state = GBPT_REQ_CANCELLED;
            r->t_done = host_clock();
        }
    }
    std::vector<std::shared_ptr<ServerReq>> dropped;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        dropped.assign(s->queued.begin(), s->queued.end());
        s->queued.clear();
        s->wake.notify_all();
        s->done.notify_all();
    }
    for (auto& r : dropped) s->release_scene(*r);
    if (s->thread.joinable()) s->thread.join();
    cudaStreamSynchronize(s->stream);
    s->engine.release();
    work_free(s->work);
    if (s->arena) cudaFree(s->arena);
    for (cudaEvent_t e : s->events) cudaEventDestroy(e);
    if (s->h_flags) cudaFreeHost(s->h_flags);
    if (s->stream) cudaStreamDestroy(s->stream);
    if (s->copy_stream) cudaStreamDestroy(s->copy_stream);
    s.reset();
}

} // namespace gbpt

using namespace gbpt;

extern "C" {

GBPT_API double gbpt_clock(void) { return host_clock(); }

GBPT_API int gbpt_server_start(gbpt_ctx* ctx, const gbpt_server_config* cfg) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (ctx->server) {
        set_error("gbpt_server_start: the server is already running");
        return GBPT_ERR_INVALID;
    }
    ServerPtr s(new Server());
    s->ctx = ctx;
    if (cfg) s->cfg = *cfg;
    if (s->cfg.wave_paths > (1ull << 24)) {
        set_error("gbpt_server_start: wave_paths above 2^24");
        return GBPT_ERR_INVALID;
    }
    size_t free_b = 0, total_b = 0;
    GBPT_CUDA_CHECK(cudaMemGetInfo(&free_b, &total_b));
    s->arena_bytes = s->cfg.arena_bytes
                         ? s->cfg.arena_bytes
                         : std::min<uint64_t>(free_b / 4, 16ull << 30);
    s->arena_bytes = align_up(s->arena_bytes);
    GBPT_CUDA_CHECK(cudaStreamCreateWithFlags(&s->stream, cudaStreamNonBlocking));
    GBPT_CUDA_CHECK(cudaStreamCreateWithFlags(&s->copy_stream, cudaStreamNonBlocking));
    GBPT_CUDA_CHECK(device_malloc((void**)&s->arena, s->arena_bytes));
    s->alloc.reset(s->arena_bytes);
    GBPT_CUDA_CHECK(cudaHostAlloc((void**)&s->h_flags, kTicksAhead * sizeof(uint32_t),
                                  cudaHostAllocDefault));
    std::memset(s->h_flags, 0, kTicksAhead * sizeof(uint32_t));
    for (int i = 0; i < kTicksAhead; ++i) {
        cudaEvent_t e;
        GBPT_CUDA_CHECK(cudaEventCreateWithFlags(&e, cudaEventDisableTiming));
        s->events.push_back(e);
    }
    s->engine.work = &s->work;
    s->engine.stream = s->stream;
    // unset: the context's tuning (gbpt_set_tuning / gbpt_autotune), else the default
    s->engine.wave = s->cfg.wave_paths
                         ? s->cfg.wave_paths
                         : (ctx->tuning.wave_paths ? ctx->tuning.wave_paths : kWavePaths);
    s->sort_override = ctx->tuning.sort_materials;
    s->engine.sched = sched_of(ctx->tuning);
    s->engine.use_graphs = s->cfg.use_graphs != 0;
    if ((rc = work_reserve(s->work, s->engine.wave, s->engine.wave)) != GBPT_OK) {
        set_error("gbpt_server_start: work buffer allocation failed");
        ServerPtr tmp = std::move(s);
        server_shutdown(tmp);
        return rc;
    }
    Server* raw = s.get();
    s->thread = std::thread([raw] { raw->run(); });
    ctx->server = std::move(s);
    return GBPT_OK;
}

GBPT_API int gbpt_server_stop(gbpt_ctx* ctx) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    ServerPtr s;
    {
        std::lock_guard<std::mutex> lk(ctx->mu);
        s = std::move(ctx->server);
    }
    if (!s) {
        set_error("gbpt_server_stop: the server is not running");
        return GBPT_ERR_INVALID;
    }
    server_shutdown(s);
    return GBPT_OK;
}

GBPT_API int gbpt_server_submit(gbpt_ctx* ctx, const gbpt_request* req, uint64_t* ticket) {
    int rc = check_ctx(ctx);
    if (rc) return rc;
    if (!req || !ticket) {
        set_error("gbpt_server_submit: null argument");
        return GBPT_ERR_INVALID;
    }
    if ((rc = validate_params(&req->camera, &req->params))) return rc;
    if (!req->out_host == !req->out_device) {
        set_error("gbpt_server_submit: exactly one of out_host and out_device must be set");
        return GBPT_ERR_INVALID;
    }
    auto r = std::make_shared<ServerReq>();
    r->req = *req;
    r->n_pix = req->params.pixel_count ? req->params.pixel_count
                                       : req->params.width * req->params.height;
    if (req->params.pixel_count)
        r->pixels.assign(req->params.pixels, req->params.pixels + req->params.pixel_count);
    r->req.params.pixels = nullptr;
    std::lock_guard<std::mutex> lk(ctx->mu);
    Server* s = ctx->server.get();
    if (!s) {
        set_error("gbpt_server_submit: the server is not running");
        return GBPT_ERR_INVALID;
    }
    auto it = ctx->scenes.find(req->scene);
    if (it == ctx->scenes.end()) {
        set_error("gbpt_server_submit: unknown scene id");
        return GBPT_ERR_NOT_FOUND;
    }
    if ((uint64_t)std::max(req->params.spp, 0) > s->engine.wave) {
        set_error("gbpt_server_submit: spp above the server's wave size");
        return GBPT_ERR_INVALID;
    }
    const uint64_t need = (req->out_host ? align_up((uint64_t)r->n_pix * 16) : 0) +
                          align_up((uint64_t)r->pixels.size() * 4);
    if (need > s->arena_bytes) {
        set_error("gbpt_server_submit: the request's output exceeds the server's output arena");
        return GBPT_ERR_NO_MEMORY;
    }
    r->scene = &it->second;
    ++ctx->scene_users[req->scene];
    {
        std::lock_guard<std::mutex> sl(s->mu);
        r->ticket = s->next_ticket++;
        r->t_submit = host_clock();
        s->all[r->ticket] = r;
        s->queued.push_back(r);
        s->wake.notify_all();
    }
    *ticket = r->ticket;
    return GBPT_OK;
}

static int status_of(const ServerReq& r, gbpt_request_status* st) {
    if (st) {
        st->state = r.state;
        st->error = r.error;
        st->submit_s = r.t_submit;
        st->admit_s = r.t_admit;
        st->done_s = r.t_done;
        st->samples = (uint64_t)r.n_pix * (uint64_t)std::max(r.req.params.spp, 0);
    }
    switch (r.state) {
    case GBPT_REQ_DONE: return GBPT_OK;
    case GBPT_REQ_CANCELLED: return GBPT_ERR_CANCELLED;
    case GBPT_REQ_FAILED: return r.error != GBPT_OK ? r.error : GBPT_ERR_CUDA;
    default: return GBPT_ERR_BUSY;
    }
}

static Server* server_of(gbpt_ctx* ctx, const char* who) {
    if (!ctx) {
        set_error("null context");
        return nullptr;
    }
    std::lock_guard<std::mutex> lk(ctx->mu);
    if (!ctx->server) set_error(std::string(who) + ": the server is not running");
    return ctx->server.get();
}

GBPT_API int gbpt_server_poll(gbpt_ctx* ctx, uint64_t ticket, gbpt_request_status* status) {
    Server* s = server_of(ctx, "gbpt_server_poll");
    if (!s) return GBPT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) {
        set_error("gbpt_server_poll: unknown ticket");
        return GBPT_ERR_NOT_FOUND;
    }
    return status_of(*it->second, status);
}

GBPT_API int gbpt_server_wait(gbpt_ctx* ctx, uint64_t ticket, double timeout_s,
                              gbpt_request_status* status) {
    Server* s = server_of(ctx, "gbpt_server_wait");
    if (!s) return GBPT_ERR_INVALID;
    std::unique_lock<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) {
        set_error("gbpt_server_wait: unknown ticket");
        return GBPT_ERR_NOT_FOUND;
    }
    std::shared_ptr<ServerReq> r = it->second;
    auto finished = [&] {
        return r->state == GBPT_REQ_DONE || r->state == GBPT_REQ_CANCELLED ||
               r->state == GBPT_REQ_FAILED;
    };
    if (timeout_s < 0) s->done.wait(lk, finished);
    else s->done.wait_for(lk, std::chrono::duration<double>(timeout_s), finished);
    return status_of(*r, status);
}

GBPT_API int gbpt_server_cancel(gbpt_ctx* ctx, uint64_t ticket) {
    Server* s = server_of(ctx, "gbpt_server_cancel");
    if (!s) return GBPT_ERR_INVALID;
    std::shared_ptr<ServerReq> dropped;
    {
        std::lock_guard<std::mutex> lk(s->mu);
        auto it = s->all.find(ticket);
        if (it == s->all.end()) {
            set_error("gbpt_server_cancel: unknown ticket");
            return GBPT_ERR_NOT_FOUND;
        }
        std::shared_ptr<ServerReq> r = it->second;
        if (r->state == GBPT_REQ_QUEUED) {
            s->queued.erase(std::remove(s->queued.begin(), s->queued.end(), r), s->queued.end());
            r->state = GBPT_REQ_CANCELLED;
            r->t_done = host_clock();
            dropped = r;
            s->done.notify_all();
        } else if (r->state == GBPT_REQ_RUNNING) {
            r->cancel = true; // stops at the next tick boundary
            s->wake.notify_all();
        }
    }
    if (dropped) s->release_scene(*dropped);
    return GBPT_OK;
}

GBPT_API int gbpt_server_release(gbpt_ctx* ctx, uint64_t ticket) {
    Server* s = server_of(ctx, "gbpt_server_release");
    if (!s) return GBPT_ERR_INVALID;
    std::lock_guard<std::mutex> lk(s->mu);
    auto it = s->all.find(ticket);
    if (it == s->all.end()) {
        set_error("gbpt_server_release: unknown ticket");
        return GBPT_ERR_NOT_FOUND;
    }
    const int st = it->second->state;
    if (st == GBPT_REQ_QUEUED || st == GBPT_REQ_RUNNING) {
        set_error("gbpt_server_release: the request has not finished");
        return GBPT_ERR_BUSY;
    }
    s->all.erase(it);
    return GBPT_OK;
}

GBPT_API int gbpt_server_info(gbpt_ctx* ctx, gbpt_server_stats* info) {
    Server* s = server_of(ctx, "gbpt_server_info");
    if (!s) return GBPT_ERR_INVALID;
    if (!info) {
        set_error("gbpt_server_info: null output");
        return GBPT_ERR_INVALID;
    }
    std::lock_guard<std::mutex> lk(s->mu);
    std::memset(info, 0, sizeof(*info));
    info->queued = s->queued.size();
    info->active = s->active.size();
    info->completed = s->completed;
    info->ticks = s->ticks;
    info->kernel_launches = s->launches;
    info->paths = s->paths;
    info->arena_bytes = s->arena_bytes;
    info->wave_paths = s->engine.wave;
    return s->fatal.empty() ? GBPT_OK : GBPT_ERR_CUDA;
}

} // extern "C"
