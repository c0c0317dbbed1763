// sgl_serve.cpp — the serving loop: render requests of different scenes and
// viewport sizes are admitted against a device-memory budget (framebuffer +
// scratch), batched as they arrive and run on several streams at once; each
// finished frame can be copied to the caller's host buffers.
//
// Continuous batching: a worker thread keeps up to `streams` batches in
// flight; whenever one finishes, its memory returns to the budget and the
// requests that arrived meanwhile form the next batch on the freed stream.
// A request with transparency layers runs as a batch of its own (its
// framebuffer is the layers' surface); when its fragment pool turns out too
// small it is launched again with a larger one before it completes.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <memory>
#include <mutex>
#include <thread>
#include <unordered_map>
#include <vector>

#include <cuda_runtime.h>

#include "sgl.h"
#include "sgl_internal.h"
#include "sgl_runtime.h"

namespace sgl {

static double now_s()
{
    using namespace std::chrono;
    return duration<double>(steady_clock::now().time_since_epoch()).count();
}

struct Job {
    uint64_t ticket;
    sgl_request req;
    Scene *scene;
    size_t bytes;
    sgl_request_result res;
    std::vector<float> pose; // a posed request: node world matrices, then the normal matrices (16 floats per node)
};

struct Server {
    Ctx *ctx = nullptr;   // the owning context (scenes); only read by the worker
    Ctx errors;           // the worker's own error sink (ctx->last_error belongs to the caller's thread)
    sgl_serve_opts opts{};
    struct LaneState {
        std::unique_ptr<Lane> lane;
        DevBuf frames; // framebuffers of the batch in flight: colour then depth per job
        DevBuf poses;  // posed requests: node matrices, world positions and normals per job
        std::vector<Job> jobs;
        size_t bytes = 0;
        int slot = 0;
        bool busy = false;
        bool layered = false; // the batch is one request with transparency layers
        // copy-out: timing events around the batch's copies to the host, so that
        // a result also says when its frame was complete on the device
        cudaEvent_t ev_rendered = nullptr, ev_copied = nullptr;
        bool timed_copy = false;
        ~LaneState()
        {
            if (ev_rendered)
                cudaEventDestroy(ev_rendered);
            if (ev_copied)
                cudaEventDestroy(ev_copied);
        }
    };
    std::vector<std::unique_ptr<LaneState>> lanes;
    std::mutex mu;
    std::condition_variable cv_submit, cv_done;
    std::deque<Job> pending;
    std::unordered_map<uint64_t, sgl_request_result> done;
    uint64_t next_ticket = 1;
    uint64_t submitted = 0, completed = 0;
    uint64_t batches = 0, kernels = 0; // launched by the worker
    size_t in_flight_bytes = 0;
    bool stop = false;
    std::thread worker;
    int tile = 16, span_bin = 16;

    void run();
    void launch_batch_on(LaneState &ls, std::vector<Job> &&jobs);
    void finish(LaneState &ls);
};

static size_t request_bytes(const Scene *s, const sgl_view &v)
{
    // layered views: a first fragment pool of 4 fragments per pixel (32 B
    // each), list heads and the merged layer (4 + 4 B per pixel)
    const size_t layers = v.layers > 0 ? 136 * (size_t)v.w * v.h : 0;
    return 8 * (size_t)v.w * v.h + view_scratch_bytes(s->n_vertices, s->n_triangles, v.w, v.h) + layers;
}

void Server::launch_batch_on(LaneState &ls, std::vector<Job> &&jobs)
{
    Ctx *c = &errors;
    size_t fb = 0;
    for (auto &j : jobs)
        fb += 8 * (size_t)j.req.view.w * j.req.view.h;
    sgl_status st = SGL_OK;
    if (ls.frames.ensure(std::max<size_t>(fb, 256)) != cudaSuccess) {
        c->fail("serving: framebuffer allocation of %zu bytes failed", fb);
        st = SGL_ERR_OOM;
    }
    // posed requests: their node matrices and world arrays, then k_pose
    auto pose_span = [](const Job &j) {
        return (sizeof(float) * j.pose.size() + 16 + 32 * (size_t)j.scene->n_vertices +
                (j.scene->dev.pbox ? 32 * (size_t)j.scene->dev.n_prims : 0) + 255) & ~(size_t)255;
    };
    size_t pose_bytes = 0;
    for (auto &j : jobs)
        if (!j.pose.empty())
            pose_bytes += pose_span(j);
    if (st == SGL_OK && pose_bytes && ls.poses.ensure(pose_bytes) != cudaSuccess) {
        c->fail("serving: pose scratch of %zu bytes failed", pose_bytes);
        st = SGL_ERR_OOM;
    }
    std::vector<BatchEntry> entries;
    entries.reserve(jobs.size());
    size_t off = 0, pose_off = 0;
    std::vector<std::pair<uint32_t *, float *>> bufs;
    for (auto &j : jobs) {
        const size_t px = (size_t)j.req.view.w * j.req.view.h;
        uint32_t *pix = (uint32_t *)((uint8_t *)ls.frames.ptr + off);
        float *z = (float *)((uint8_t *)ls.frames.ptr + off + 4 * px);
        off += 8 * px;
        sgl_view v = j.req.view;
        v.x = 0;
        v.y = 0;
        entries.push_back(BatchEntry{j.scene, v, pix, v.w, z});
        entries.back().surface = pix; // a layered request's surface is its own framebuffer
        bufs.emplace_back(pix, z);
        if (!j.pose.empty() && st == SGL_OK) {
            uint8_t *base = (uint8_t *)ls.poses.ptr + pose_off;
            float *mats = (float *)base;
            const size_t nm = j.pose.size() / 2;
            float4 *wpos = (float4 *)(base + ((sizeof(float) * j.pose.size() + 15) & ~(size_t)15));
            float4 *wnrm = wpos + j.scene->n_vertices;
            float4 *pbox = j.scene->dev.pbox ? wnrm + j.scene->n_vertices : nullptr; // (2 per primitive)
            pose_off += pose_span(j);
            if (cudaMemcpyAsync(mats, j.pose.data(), sizeof(float) * j.pose.size(), cudaMemcpyHostToDevice,
                                ls.lane->stream) != cudaSuccess ||
                launch_pose(j.scene->dev, mats, mats + nm, wpos, wnrm, pbox, ls.lane->stream) != cudaSuccess) {
                c->fail("serving: pose of request %llu failed", (unsigned long long)j.ticket);
                st = SGL_ERR_CUDA;
            }
            entries.back().wpos = wpos;
            entries.back().wnrm = wnrm;
            entries.back().pbox = pbox;
            entries.back().node_world = mats;
            entries.back().node_rs = mats + nm;
        }
    }
    ls.layered = jobs.size() == 1 && jobs[0].req.view.layers > 0;
    const double t0 = now_s();
    if (st == SGL_OK)
        st = ls.lane->prepare(c, entries.data(), (int)entries.size(), tile, span_bin, nullptr, &ls.slot);
    int kernels_launched = 0;
    if (st == SGL_OK)
        st = ls.lane->launch(c, ls.slot, tile, !ls.layered, &kernels_launched, nullptr);
    {
        std::lock_guard<std::mutex> g(mu);
        batches++;
        kernels += (uint64_t)kernels_launched;
    }
    if (st == SGL_OK && opts.copy_out) {
        // colour then depth of each request, in framebuffer order; copies whose
        // host and device ranges both continue the previous one are merged (a
        // caller whose host buffers follow the same layout gets one copy per batch)
        struct Span {
            uint8_t *dst;
            const uint8_t *src;
            size_t n;
        };
        std::vector<Span> spans;
        spans.reserve(2 * jobs.size());
        auto add = [&](void *dst, const void *src, size_t n) {
            if (!dst)
                return;
            if (!spans.empty()) {
                Span &b = spans.back();
                if (b.dst + b.n == (uint8_t *)dst && b.src + b.n == (const uint8_t *)src) {
                    b.n += n;
                    return;
                }
            }
            spans.push_back(Span{(uint8_t *)dst, (const uint8_t *)src, n});
        };
        for (size_t i = 0; i < jobs.size(); i++) {
            const size_t px = (size_t)jobs[i].req.view.w * jobs[i].req.view.h;
            add(jobs[i].req.host_pixels, bufs[i].first, 4 * px);
            add(jobs[i].req.host_zbuffer, bufs[i].second, 4 * px);
        }
        bool issued = false;
        ls.timed_copy = ls.ev_rendered && ls.ev_copied &&
                        cudaEventRecord(ls.ev_rendered, ls.lane->stream) == cudaSuccess;
        for (const Span &sp : spans) {
            if (cudaMemcpyAsync(sp.dst, sp.src, sp.n, cudaMemcpyDeviceToHost, ls.lane->stream) != cudaSuccess) {
                cudaGetLastError(); // reported through the requests' status, not a later call
                st = SGL_ERR_CUDA;
                break;
            }
            issued = true;
        }
        // the lane's done event must come after every copy that was issued, so
        // that no request is reported done while its host buffers are written
        if (issued && cudaEventRecord(ls.lane->slots[ls.slot].done, ls.lane->stream) != cudaSuccess) {
            cudaGetLastError();
            st = SGL_ERR_CUDA;
        }
        if (ls.timed_copy && cudaEventRecord(ls.ev_copied, ls.lane->stream) != cudaSuccess) {
            cudaGetLastError();
            ls.timed_copy = false;
        }
    } else {
        ls.timed_copy = false;
    }
    for (auto &j : jobs) {
        j.res.start_s = t0;
        j.res.status = st;
    }
    ls.jobs = std::move(jobs);
    ls.busy = true;
}

void Server::finish(LaneState &ls)
{
    if (ls.layered && !ls.jobs.empty() && ls.jobs[0].res.status == SGL_OK) {
        bool fit = true;
        const sgl_status st = ls.lane->layered_fit(&errors, ls.slot, &fit);
        if (st == SGL_OK && !fit) {
            // the fragment pool grew: render the request again (nothing was written)
            std::vector<Job> again = std::move(ls.jobs);
            launch_batch_on(ls, std::move(again));
            return;
        }
        if (st != SGL_OK)
            ls.jobs[0].res.status = st;
    }
    std::vector<unsigned long long> per_item;
    sgl_status st = ls.lane->read_counters(&errors, ls.slot, nullptr, nullptr, &per_item);
    const double t = now_s();
    double copy_s = 0.0; // device time of the batch's copies to the host
    if (ls.timed_copy) {
        float ms = 0.0f;
        if (cudaEventSynchronize(ls.ev_copied) == cudaSuccess &&
            cudaEventElapsedTime(&ms, ls.ev_rendered, ls.ev_copied) == cudaSuccess && ms > 0.0f)
            copy_s = 1e-3 * (double)ms;
        else
            cudaGetLastError();
        ls.timed_copy = false;
    }
    std::lock_guard<std::mutex> g(mu);
    for (size_t i = 0; i < ls.jobs.size(); i++) {
        Job &j = ls.jobs[i];
        j.res.done_s = t;
        j.res.rendered_s = t - copy_s;
        if (j.res.status == SGL_OK)
            j.res.status = st;
        j.res.fragments = (2 * i + 1 < per_item.size()) ? per_item[2 * i + 1] : 0;
        done[j.ticket] = j.res;
        in_flight_bytes -= j.bytes;
        completed++;
    }
    ls.jobs.clear();
    ls.busy = false;
    cv_done.notify_all();
}

void Server::run()
{
    cudaSetDevice(ctx->device);
    for (;;) {
        // completions
        for (auto &lp : lanes) {
            LaneState &ls = *lp;
            if (ls.busy) {
                cudaError_t q = cudaEventQuery(ls.lane->slots[ls.slot].done);
                if (q == cudaSuccess)
                    finish(ls);
                else if (q != cudaErrorNotReady) {
                    cudaGetLastError();
                    for (auto &j : ls.jobs)
                        j.res.status = SGL_ERR_CUDA;
                    finish(ls);
                }
            }
        }
        // admission: the requests that fit the budget, in arrival order, to a free stream
        LaneState *free_lane = nullptr;
        for (auto &lp : lanes)
            if (!lp->busy) {
                free_lane = lp.get();
                break;
            }
        std::vector<Job> batch;
        {
            std::unique_lock<std::mutex> lk(mu);
            if (stop && pending.empty()) {
                bool any_busy = false;
                for (auto &lp : lanes)
                    any_busy |= lp->busy;
                if (!any_busy)
                    return;
            }
            if (free_lane) {
                while (!pending.empty() && (int)batch.size() < opts.max_batch) {
                    Job &j = pending.front();
                    const bool layered = j.req.view.layers > 0;
                    if (layered && !batch.empty())
                        break; // a layered request runs alone
                    if (in_flight_bytes + j.bytes > opts.budget_bytes && !(batch.empty() && in_flight_bytes == 0))
                        break; // wait for memory; a lone request larger than what is free still runs alone
                    in_flight_bytes += j.bytes;
                    batch.push_back(j);
                    pending.pop_front();
                    if (layered)
                        break;
                }
            }
            if (batch.empty()) {
                bool any_busy = false;
                for (auto &lp : lanes)
                    any_busy |= lp->busy;
                if (!any_busy || !free_lane)
                    cv_submit.wait_for(lk, std::chrono::microseconds(any_busy ? 20 : 2000));
                else
                    cv_submit.wait_for(lk, std::chrono::microseconds(20));
                continue;
            }
        }
        launch_batch_on(*free_lane, std::move(batch));
    }
}

} // namespace sgl

using namespace sgl;

extern "C" {

SGL_API sgl_status sgl_server_create(sgl_ctx *c, const sgl_serve_opts *opts, sgl_server **out)
{
    Ctx *ctx = reinterpret_cast<Ctx *>(c);
    if (!ctx || !out)
        return SGL_ERR_INVALID;
    *out = nullptr;
    cudaSetDevice(ctx->device);
    auto *srv = new (std::nothrow) Server();
    if (!srv)
        return SGL_ERR_OOM;
    srv->ctx = ctx;
    srv->errors.device = ctx->device;
    srv->opts = opts ? *opts : sgl_serve_opts{};
    if (srv->opts.budget_bytes == 0)
        srv->opts.budget_bytes = 40ull << 30;
    if (srv->opts.max_batch <= 0 || srv->opts.max_batch > kMaxBatch)
        srv->opts.max_batch = 64;
    if (srv->opts.streams <= 0 || srv->opts.streams > 16)
        srv->opts.streams = 3;
    srv->tile = ctx->tile;
    srv->span_bin = ctx->inline_span;
    for (int i = 0; i < srv->opts.streams; i++) {
        srv->lanes.push_back(std::make_unique<Server::LaneState>());
        Server::LaneState &ls = *srv->lanes.back();
        ls.lane = std::make_unique<Lane>();
        // blocking streams: work on the legacy default stream (a caller's timing
        // events) is ordered with every batch
        sgl_status st = ls.lane->init(&srv->errors, srv->opts.max_batch, nullptr, true);
        if (st != SGL_OK) {
            delete srv;
            return st;
        }
        if (srv->opts.copy_out && (cudaEventCreate(&ls.ev_rendered) != cudaSuccess ||
                                   cudaEventCreate(&ls.ev_copied) != cudaSuccess)) {
            cudaGetLastError(); // results then carry rendered_s = done_s
            ls.ev_rendered = ls.ev_copied = nullptr;
        }
    }
    srv->worker = std::thread([srv] { srv->run(); });
    *out = reinterpret_cast<sgl_server *>(srv);
    return SGL_OK;
}

// A request checked and turned into a job (nothing queued yet).
static sgl_status make_job(Server *srv, const sgl_request *req, Job &j)
{
    Scene *scene = srv->ctx->find(req->scene_id);
    if (!scene)
        return SGL_ERR_NOT_FOUND;
    const sgl_view &v = req->view;
    if (v.w <= 0 || v.h <= 0 || (int64_t)v.w * v.h > (1ll << 28) || v.layers < 0 || v.layers > SGL_MAX_LAYERS)
        return SGL_ERR_INVALID;
    if (v.dof.enabled && !(v.dof.max_radius >= 0.0f && v.dof.max_radius <= 4096.0f))
        return SGL_ERR_INVALID;
    j = Job{};
    j.req = *req;
    j.scene = scene;
    j.bytes = request_bytes(scene, v);
    if (req->nodes) {
        if (req->n_nodes != (int)scene->nodes.size())
            return SGL_ERR_INVALID; // a pose gives every node of the scene
        std::vector<sgl_node_desc> nd(req->nodes, req->nodes + req->n_nodes);
        std::vector<float> world, rs;
        if (!node_matrices(nd, world, rs))
            return SGL_ERR_INVALID;
        j.pose = std::move(world);
        j.pose.insert(j.pose.end(), rs.begin(), rs.end());
        j.bytes += sizeof(float) * j.pose.size() + 32 * (size_t)scene->n_vertices + 512;
    }
    j.req.nodes = nullptr; // copied
    if (j.bytes > srv->opts.budget_bytes)
        return SGL_ERR_BUDGET;
    j.res.submit_s = now_s();
    j.res.status = SGL_ERR_BUSY;
    return SGL_OK;
}

SGL_API sgl_status sgl_server_submit(sgl_server *s, const sgl_request *req, uint64_t *ticket)
{
    Server *srv = reinterpret_cast<Server *>(s);
    if (!srv || !req || !ticket)
        return SGL_ERR_INVALID;
    Job j;
    const sgl_status st = make_job(srv, req, j);
    if (st != SGL_OK)
        return st;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        if (srv->stop)
            return SGL_ERR_INVALID;
        j.ticket = srv->next_ticket++;
        srv->pending.push_back(std::move(j));
        srv->submitted++;
        *ticket = srv->pending.back().ticket;
    }
    srv->cv_submit.notify_one();
    return SGL_OK;
}

SGL_API sgl_status sgl_server_submit_batch(sgl_server *s, const sgl_request *reqs, int n, uint64_t *tickets,
                                           int *n_queued)
{
    Server *srv = reinterpret_cast<Server *>(s);
    if (n_queued)
        *n_queued = 0;
    if (!srv || n < 0 || (n > 0 && (!reqs || !tickets)))
        return SGL_ERR_INVALID;
    sgl_status st = SGL_OK;
    int k = 0;
    std::vector<Job> jobs;
    jobs.reserve((size_t)n);
    for (; k < n; k++) {
        Job j;
        st = make_job(srv, reqs + k, j);
        if (st != SGL_OK)
            break;
        jobs.push_back(std::move(j));
    }
    {
        std::lock_guard<std::mutex> g(srv->mu);
        if (srv->stop)
            return SGL_ERR_INVALID;
        for (size_t i = 0; i < jobs.size(); i++) {
            jobs[i].ticket = srv->next_ticket++;
            tickets[i] = jobs[i].ticket;
            srv->pending.push_back(std::move(jobs[i]));
            srv->submitted++;
        }
    }
    if (k > 0)
        srv->cv_submit.notify_one();
    if (n_queued)
        *n_queued = k;
    return st;
}

SGL_API sgl_status sgl_server_poll(sgl_server *s, uint64_t ticket, sgl_request_result *result)
{
    Server *srv = reinterpret_cast<Server *>(s);
    if (!srv)
        return SGL_ERR_INVALID;
    std::lock_guard<std::mutex> g(srv->mu);
    auto it = srv->done.find(ticket);
    if (it == srv->done.end())
        return (ticket == 0 || ticket >= srv->next_ticket) ? SGL_ERR_NOT_FOUND : SGL_ERR_BUSY;
    if (result)
        *result = it->second;
    srv->done.erase(it);
    return SGL_OK;
}

SGL_API sgl_status sgl_server_wait(sgl_server *s, uint64_t ticket, double timeout_s, sgl_request_result *result)
{
    Server *srv = reinterpret_cast<Server *>(s);
    if (!srv)
        return SGL_ERR_INVALID;
    std::unique_lock<std::mutex> lk(srv->mu);
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    for (;;) {
        auto it = srv->done.find(ticket);
        if (it != srv->done.end()) {
            if (result)
                *result = it->second;
            srv->done.erase(it);
            return SGL_OK;
        }
        if (ticket == 0 || ticket >= srv->next_ticket)
            return SGL_ERR_NOT_FOUND;
        if (srv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout)
            return SGL_ERR_TIMEOUT;
    }
}

SGL_API sgl_status sgl_server_wait_batch(sgl_server *s, const uint64_t *tickets, int n, double timeout_s,
                                         sgl_request_result *results)
{
    Server *srv = reinterpret_cast<Server *>(s);
    if (!srv || n < 0 || (n > 0 && !tickets))
        return SGL_ERR_INVALID;
    std::unique_lock<std::mutex> lk(srv->mu);
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    for (int i = 0; i < n; i++) {
        const uint64_t ticket = tickets[i];
        for (;;) {
            auto it = srv->done.find(ticket);
            if (it != srv->done.end()) {
                if (results)
                    results[i] = it->second;
                srv->done.erase(it);
                break;
            }
            if (ticket == 0 || ticket >= srv->next_ticket)
                return SGL_ERR_NOT_FOUND;
            if (srv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout)
                return SGL_ERR_TIMEOUT;
        }
    }
    return SGL_OK;
}

SGL_API sgl_status sgl_server_drain(sgl_server *s, double timeout_s)
{
    Server *srv = reinterpret_cast<Server *>(s);
    if (!srv)
        return SGL_ERR_INVALID;
    std::unique_lock<std::mutex> lk(srv->mu);
    const auto deadline = std::chrono::steady_clock::now() + std::chrono::duration<double>(timeout_s);
    while (srv->completed < srv->submitted)
        if (srv->cv_done.wait_until(lk, deadline) == std::cv_status::timeout)
            return SGL_ERR_TIMEOUT;
    return SGL_OK;
}

SGL_API sgl_status sgl_server_stats(sgl_server *s, uint64_t *batches, uint64_t *kernels, uint64_t *completed)
{
    Server *srv = reinterpret_cast<Server *>(s);
    if (!srv)
        return SGL_ERR_INVALID;
    std::lock_guard<std::mutex> g(srv->mu);
    if (batches)
        *batches = srv->batches;
    if (kernels)
        *kernels = srv->kernels;
    if (completed)
        *completed = srv->completed;
    return SGL_OK;
}

SGL_API void sgl_server_destroy(sgl_server *s)
{
    Server *srv = reinterpret_cast<Server *>(s);
    if (!srv)
        return;
    {
        std::lock_guard<std::mutex> g(srv->mu);
        srv->stop = true;
    }
    srv->cv_submit.notify_all();
    if (srv->worker.joinable())
        srv->worker.join();
    delete srv;
}

} // extern "C"
