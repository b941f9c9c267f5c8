// Serving loop: continuous batching of render requests over resident scenes.
//
// A server thread owns two wave lanes (a stream and wave buffers each), a device
// job table with one slot per admitted request and an arena for per-request state
// (per-pixel sums, and film staging for host films). Each iteration it
//   1. admits queued requests while slots and arena space are free,
//   2. packs the next sample blocks of the admitted requests into one wave,
//      least remaining work first (a short request that arrives behind a long
//      one finishes in the next wave; the long one takes what is left),
//   3. enqueues the wave and the finalization of the requests it completes on
//      the lane the wave before last used, then retires the previous wave.
// Consecutive waves run on the two lanes, so a wave starts while the one before
// it finishes its last, sparse bounces; each wave accumulates only after the one
// before it has accumulated and finalised (an event chain). Requests that arrive
// while a wave runs join the next one. A request's film does not depend on the
// mix or the lanes: paths draw from a stream keyed by (seed, pixel, sample) and
// each pixel sums its samples in sample order.
#include <algorithm>
#include <chrono>
#include <condition_variable>
#include <deque>
#include <map>
#include <thread>

#include "context.h"

namespace ptg {

namespace {
using Clock = std::chrono::steady_clock;

struct Request {
    uint64_t id = 0;
    pt_job job{};
    float* filmHost = nullptr;
    SceneGpu* scene = nullptr;
    int state = PT_REQ_QUEUED;
    int status = PT_OK;
    double submit = 0, admit = -1, done = -1;
    int pixels = 0, spp = 0;
    int scheduled = 0, finished = 0;  // samples put in waves / completed
    int slot = -1;
    size_t accumOff = 0, accumBytes = 0, filmOff = 0, filmBytes = 0;
    int inFlight = 0;  // waves holding this request's samples
    bool cancel = false;
    double deadline = 0;    // seconds since the server started; 0: none
    bool timedOut = false;  // cancelled by its deadline (fails with PT_ERR_TIMEOUT)
};
}  // namespace

class Server {
public:
    Server(pt_context* ctx, const pt_serve_config& cfg) : ctx_(ctx), cfg_(cfg) {
        // 2^26 paths (15.8 GB of wave state per lane): at saturation the waves are full
        // enough to beat one-request-at-a-time rendering; under light load they stay small
        if (cfg_.wave_paths <= 0) cfg_.wave_paths = 1 << 26;
        if (cfg_.max_active <= 0) cfg_.max_active = 256;
        cfg_.max_active = std::min(cfg_.max_active, kMaxJobsPerCall);
        if (cfg_.state_budget == 0) cfg_.state_budget = uint64_t(4) << 30;
    }
    ~Server() { Stop(); }

    int Start() {  // ctx->mu held by the caller
        for (cudaStream_t& s : stream_) {
            const cudaError_t e = cudaStreamCreateWithFlags(&s, cudaStreamNonBlocking);
            if (e != cudaSuccess) {
                DestroyStreams();
                return CudaFail(ctx_, e, "server stream");
            }
        }
        int rc;
        if ((rc = Alloc(ctx_, arena_, cfg_.state_budget)) != PT_OK ||
            (rc = Alloc(ctx_, jobTable_, sizeof(DevJob) * cfg_.max_active)) != PT_OK ||
            (rc = Alloc(ctx_, units_[0], sizeof(WaveUnit) * kMaxUnitsPerWave)) != PT_OK ||
            (rc = Alloc(ctx_, units_[1], sizeof(WaveUnit) * kMaxUnitsPerWave)) != PT_OK ||
            (rc = Alloc(ctx_, jobList_[0], sizeof(int) * cfg_.max_active)) != PT_OK ||
            (rc = Alloc(ctx_, jobList_[1], sizeof(int) * cfg_.max_active)) != PT_OK ||
            (rc = AllocWave()) != PT_OK) {
            FreeAll();
            DestroyStreams();
            return rc;
        }
        alloc_.Reset(cfg_.state_budget);
        tune_ = ctx_->tuning;
        graphs_ = NewWaveGraphCache();
        slotJobs_.assign(cfg_.max_active, DevJob{});
        for (int s = cfg_.max_active - 1; s >= 0; s--) freeSlots_.push_back(s);
        t0_ = Clock::now();
        thread_ = std::thread([this] { Loop(); });
        return PT_OK;
    }

    int Submit(const pt_job* job, float* filmHost, uint64_t* id) {
        const double submitted = Now();
        SceneGpu* sg = nullptr;
        {
            std::lock_guard<std::mutex> g(ctx_->mu);
            const int rc = CheckArgs(ctx_, job->scene, &job->camera, &job->settings, &sg);
            if (rc != PT_OK) return rc;
            if (job->settings.mode != PT_MODE_WAVEFRONT)
                return Fail(ctx_, PT_ERR_INVALID_ARG, "served renders use the wavefront mode");
            if (!filmHost && !job->film_device)
                return Fail(ctx_, PT_ERR_INVALID_ARG, "a device or host film is required");
            sg->refs++;
        }
        auto r = std::make_unique<Request>();
        r->job = *job;
        r->filmHost = filmHost;
        r->scene = sg;
        r->pixels = job->settings.width * job->settings.height;
        r->spp = job->settings.spp;
        r->accumBytes = sizeof(float4) * (size_t)r->pixels;
        r->filmBytes = filmHost ? sizeof(float) * 3 * (size_t)r->pixels : 0;
        if (r->pixels > cfg_.wave_paths ||
            ((r->accumBytes + 255) & ~size_t(255)) + ((r->filmBytes + 255) & ~size_t(255)) >
              cfg_.state_budget) {
            sg->refs--;
            return Fail(ctx_, PT_ERR_OVER_BUDGET, "request exceeds the wave or the state budget");
        }
        std::lock_guard<std::mutex> g(mu_);
        if (stopping_) {
            sg->refs--;
            return Fail(ctx_, PT_ERR_BUSY, "server is stopping");
        }
        r->id = nextId_++;
        r->submit = submitted;
        *id = r->id;
        queue_.push_back(r->id);
        reqs_[r->id] = std::move(r);
        cv_.notify_all();
        return PT_OK;
    }

    int Poll(uint64_t id, pt_request_status* out) {
        std::lock_guard<std::mutex> g(mu_);
        return Fill(id, out);
    }

    int Wait(uint64_t id, double timeout, pt_request_status* out) {
        std::unique_lock<std::mutex> lk(mu_);
        auto it = reqs_.find(id);
        if (it == reqs_.end()) return PT_ERR_NOT_FOUND;
        const bool ok = doneCv_.wait_for(lk, std::chrono::duration<double>(timeout), [&] {
            const int s = it->second->state;
            return s == PT_REQ_DONE || s == PT_REQ_CANCELLED || s == PT_REQ_FAILED;
        });
        Fill(id, out);
        return ok ? PT_OK : PT_ERR_TIMEOUT;
    }

    int Cancel(uint64_t id) {
        std::lock_guard<std::mutex> g(mu_);
        auto it = reqs_.find(id);
        if (it == reqs_.end()) return PT_ERR_NOT_FOUND;
        it->second->cancel = true;
        cv_.notify_all();
        return PT_OK;
    }

    // seconds after submission; 0 clears
    int SetDeadline(uint64_t id, double seconds) {
        std::lock_guard<std::mutex> g(mu_);
        auto it = reqs_.find(id);
        if (it == reqs_.end()) return PT_ERR_NOT_FOUND;
        Request& r = *it->second;
        if (r.state != PT_REQ_QUEUED && r.state != PT_REQ_RUNNING) return PT_ERR_BUSY;
        r.deadline = seconds > 0.0 ? r.submit + seconds : 0.0;
        cv_.notify_all();
        return PT_OK;
    }

    int Release(uint64_t id) {
        std::lock_guard<std::mutex> g(mu_);
        auto it = reqs_.find(id);
        if (it == reqs_.end()) return PT_ERR_NOT_FOUND;
        const int s = it->second->state;
        if (s == PT_REQ_QUEUED || s == PT_REQ_RUNNING) return PT_ERR_BUSY;
        reqs_.erase(it);
        return PT_OK;
    }

    void Stop() {
        {
            std::lock_guard<std::mutex> g(mu_);
            stopping_ = true;
            cv_.notify_all();
        }
        if (thread_.joinable()) thread_.join();
        std::lock_guard<std::mutex> g(mu_);
        for (auto& kv : reqs_) {
            Request& r = *kv.second;
            if (r.state == PT_REQ_QUEUED || r.state == PT_REQ_RUNNING) Finish(r, PT_REQ_CANCELLED, PT_OK);
        }
        doneCv_.notify_all();
        if (stream_[0]) {
            std::lock_guard<std::mutex> cg(ctx_->mu);
            DestroyStreams();
            FreeAll();
        }
    }

private:
    double Now() const { return std::chrono::duration<double>(Clock::now() - t0_).count(); }

    int Fill(uint64_t id, pt_request_status* out) {
        auto it = reqs_.find(id);
        if (it == reqs_.end()) return PT_ERR_NOT_FOUND;
        const Request& r = *it->second;
        out->state = r.state;
        out->status = r.status;
        out->submit_s = r.submit;
        out->admit_s = r.admit;
        out->done_s = r.done;
        out->samples_done = (uint32_t)r.finished;
        out->samples_total = (uint32_t)r.spp;
        return PT_OK;
    }

    // mu_ held. Releases the request's slot and arena space.
    void FinishCancelled(Request& r) {
        if (r.timedOut) Finish(r, PT_REQ_FAILED, PT_ERR_TIMEOUT);
        else Finish(r, PT_REQ_CANCELLED, PT_OK);
    }

    void Finish(Request& r, int state, int status) {
        r.state = state;
        r.status = status;
        r.done = Now();
        if (r.slot >= 0) {
            alloc_.Release(r.accumOff, r.accumBytes);
            if (r.filmBytes) alloc_.Release(r.filmOff, r.filmBytes);
            freeSlots_.push_back(r.slot);
            r.slot = -1;
        }
        active_.erase(std::remove(active_.begin(), active_.end(), r.id), active_.end());
        if (r.scene) {
            r.scene->refs--;
            r.scene = nullptr;
        }
    }

    // Waits for and destroys the lanes' streams (ctx->mu held, or before the thread runs).
    void DestroyStreams() {
        for (cudaStream_t& s : stream_) {
            if (!s) continue;
            cudaStreamSynchronize(s);
            cudaStreamDestroy(s);
            s = nullptr;
        }
    }

    int AllocWave() {  // one wave of wave_paths paths per lane (streams created)
        wbBufs_.assign(2, DeviceBuffer{});
        int* host = nullptr;
        const cudaError_t e = cudaMallocHost(&host, sizeof(int) * 4);
        if (e != cudaSuccess) return CudaFail(ctx_, e, "cudaMallocHost");
        hostCount_ = host;
        for (int k = 0; k < 2; k++) {
            const int rc = Alloc(ctx_, wbBufs_[k], WaveBuffersBytes(cfg_.wave_paths));
            if (rc != PT_OK) return rc;
            wb_[k] = CarveWaveBuffers(wbBufs_[k].ptr, cfg_.wave_paths);
            wb_[k].hostCount = host + k;
            const cudaError_t z = cudaMemsetAsync(wb_[k].counts, 0, 16 * sizeof(int), stream_[k]);
            if (z != cudaSuccess) return CudaFail(ctx_, z, "wave counters");
        }
        return PT_OK;
    }

    void FreeAll() {  // ctx->mu held
        FreeWaveGraphCache(graphs_);
        graphs_ = nullptr;
        for (auto& b : wbBufs_) Free(ctx_, b);
        wbBufs_.clear();
        if (hostCount_) cudaFreeHost(hostCount_);
        hostCount_ = nullptr;
        for (WaveBuffers& w : wb_) w.hostCount = nullptr;
        Free(ctx_, arena_);
        Free(ctx_, jobTable_);
        for (int k = 0; k < 2; k++) {
            Free(ctx_, units_[k]);
            Free(ctx_, jobList_[k]);
        }
    }

    // One planned and enqueued wave: what it did, to retire once its event fires.
    struct InFlight {
        cudaEvent_t setup = nullptr;  // its job entries and sums are in place
        cudaEvent_t done = nullptr;   // accumulated, finalised, films copied
        int64_t paths = 0;  // paths the wave traces (for the throughput estimate)
        std::vector<std::pair<Request*, int>> scheduled;  // request, samples in this wave
        std::vector<Request*> finishing;
        cudaError_t error = cudaSuccess;
    };

    // mu_ held. Admits queued requests in arrival order while a slot and arena
    // space are free; returns the admitted ones (their job entries go to the device
    // with the next wave).
    std::vector<Request*> Admit() {
        std::vector<Request*> admitted;
        // requests past their deadline stop taking samples and fail once their waves retire
        const double now = Now();
        for (uint64_t id : active_) {
            Request& r = *reqs_[id];
            if (r.deadline > 0.0 && now > r.deadline && !r.cancel) r.cancel = r.timedOut = true;
        }
        for (uint64_t id : queue_) {
            Request& r = *reqs_[id];
            if (r.deadline > 0.0 && now > r.deadline && !r.cancel) r.cancel = r.timedOut = true;
        }
        for (uint64_t id : std::vector<uint64_t>(active_)) {
            Request& r = *reqs_[id];
            if (r.cancel && r.inFlight == 0) FinishCancelled(r);
        }
        for (auto it = queue_.begin(); it != queue_.end();) {
            Request& r = *reqs_[*it];
            if (r.cancel) {
                FinishCancelled(r);
                it = queue_.erase(it);
            } else {
                ++it;
            }
        }
        while (!queue_.empty() && !freeSlots_.empty()) {
            Request& r = *reqs_[queue_.front()];
            size_t off = 0, foff = 0;
            if (!alloc_.Alloc(r.accumBytes, &off)) break;
            if (r.filmBytes && !alloc_.Alloc(r.filmBytes, &foff)) {
                alloc_.Release(off, r.accumBytes);
                break;
            }
            r.accumOff = off;
            r.filmOff = foff;
            r.slot = freeSlots_.back();
            freeSlots_.pop_back();
            r.state = PT_REQ_RUNNING;
            r.admit = Now();
            active_.push_back(r.id);
            queue_.pop_front();
            admitted.push_back(&r);
        }
        return admitted;
    }

    // mu_ held. Packs the next sample blocks into a wave (PlanServeWave: least remaining
    // work first, overdue requests guaranteed their share) and records them.
    void Plan(std::vector<WaveUnit>* units, InFlight* w, int* paths, int* pixels) {
        std::vector<Request*> cand;
        std::vector<ServeRequestView> views;
        for (uint64_t id : active_) {
            Request& r = *reqs_[id];
            if (r.cancel || r.scheduled >= r.spp) continue;
            cand.push_back(&r);
            views.push_back({r.pixels, r.spp, r.scheduled, r.submit});
        }
        const ServePlanLimits lim{cfg_.wave_paths, kMaxUnitsPerWave, Now(), rate_.Rate(),
                                  kOverdueWaves, kOverdueFactor, kOverdueShare};
        for (const ServePick& p : PlanServeWave(views, lim)) {
            Request* r = cand[p.request];
            WaveUnit u{};
            u.job = r->slot;
            u.s0 = r->scheduled;
            u.sw = p.sw;
            u.pathBase = *paths;
            u.pixelBase = *pixels;
            units->push_back(u);
            *paths += r->pixels * p.sw;
            w->paths += (int64_t)r->pixels * p.sw;
            *pixels += r->pixels;
            r->scheduled += p.sw;
            r->inFlight++;
            w->scheduled.push_back({r, p.sw});
            if (r->scheduled == r->spp) w->finishing.push_back(r);
        }
    }

    // ctx->mu held. Enqueues, on the next lane, the admitted requests' job entries, the
    // wave, its accumulation (after the previous wave's) and the finalization of the
    // requests whose last samples it holds, and records the wave's events.
    cudaError_t Enqueue(const std::vector<Request*>& admitted, const std::vector<WaveUnit>& units,
                        int paths, int pixels, InFlight* w, int* launches) {
        const int lane = (int)(seq_++ & 1);
        cudaStream_t s = stream_[lane];
        cudaError_t e = cudaSuccess;
        // the other lane's latest job entries before this wave reads the table
        if (lastSetup_) e = cudaStreamWaitEvent(s, lastSetup_, 0);
        for (Request* r : admitted) {
            DevJob& J = slotJobs_[r->slot];
            J = DevJob{};
            J.S = JobScene(*r->scene, &r->job.settings);
            J.C = ToDev(&r->job.camera);
            J.st = ToDev(&r->job.settings);
            J.accum = (float4*)((char*)arena_.ptr + r->accumOff);
            J.film = r->filmHost ? (float*)((char*)arena_.ptr + r->filmOff) : r->job.film_device;
            if (e == cudaSuccess)
                e = cudaMemcpyAsync((DevJob*)jobTable_.ptr + r->slot, &J, sizeof(DevJob),
                                    cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess) e = cudaMemsetAsync(J.accum, 0, r->accumBytes, s);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->setup, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(w->setup, s);
        WaveUnit* table = (WaveUnit*)units_[lane].ptr;
        if (e == cudaSuccess && !units.empty()) {
            WaveShape shape;
            shape.nUnits = (int)units.size();
            shape.nPaths = paths;
            shape.nPixelUnits = pixels;
            shape.iters = WaveIterations(slotJobs_, units);
            shape.integrator = WaveIntegrator(slotJobs_, units);
            shape.soleJob = WaveSoleJob(units);
            shape.areaLights = WaveAreaLights(slotJobs_, units);
            std::vector<WaveUnit> ordered = units;  // rasterised units last
            PrepareRasterUnits(slotJobs_, &ordered, &shape, tune_.primaryTraversal);
            e = cudaMemcpyAsync(table, ordered.data(), ordered.size() * sizeof(WaveUnit),
                                cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess)
                e = RunWave((DevJob*)jobTable_.ptr, table, shape, wb_[lane], s, launches, nullptr, tune_,
                            graphs_, lane, false);
        }
        // sums in wave order: this wave accumulates after the previous one has
        if (e == cudaSuccess && lastDone_) e = cudaStreamWaitEvent(s, lastDone_, 0);
        if (e == cudaSuccess && !units.empty())
            e = AccumulateWave((DevJob*)jobTable_.ptr, table, wb_[lane], tune_, s, launches);
        if (e == cudaSuccess && !w->finishing.empty()) {
            std::vector<int> slots;
            int maxPx = 0;
            for (Request* r : w->finishing) {
                slots.push_back(r->slot);
                maxPx = std::max(maxPx, r->pixels);
            }
            e = cudaMemcpyAsync(jobList_[lane].ptr, slots.data(), slots.size() * sizeof(int),
                                cudaMemcpyHostToDevice, s);
            if (e == cudaSuccess)
                e = FinalizeJobs((DevJob*)jobTable_.ptr, (int*)jobList_[lane].ptr, (int)slots.size(),
                                 maxPx, s, launches, nullptr);
            for (Request* r : w->finishing)
                if (e == cudaSuccess && r->filmHost)
                    e = cudaMemcpyAsync(r->filmHost, (char*)arena_.ptr + r->filmOff, r->filmBytes,
                                        cudaMemcpyDeviceToHost, s);
        }
        if (e == cudaSuccess) e = cudaEventCreateWithFlags(&w->done, cudaEventDisableTiming);
        if (e == cudaSuccess) e = cudaEventRecord(w->done, s);
        if (e == cudaSuccess) {
            lastSetup_ = w->setup;
            lastDone_ = w->done;
        }
        return e;
    }

    // Waits for the oldest wave in flight and retires it.
    void Retire(std::deque<InFlight>& flight) {
        InFlight w = std::move(flight.front());
        flight.pop_front();
        cudaError_t e = w.error;
        if (e == cudaSuccess) e = cudaEventSynchronize(w.done);
        // a retired wave's events have fired: later waves need not wait for them
        if (lastSetup_ == w.setup) lastSetup_ = nullptr;
        if (lastDone_ == w.done) lastDone_ = nullptr;
        if (w.setup) cudaEventDestroy(w.setup);
        if (w.done) cudaEventDestroy(w.done);
        std::lock_guard<std::mutex> g(mu_);
        rate_.Retired(Now(), w.paths, e == cudaSuccess, !flight.empty());
        for (auto& [r, sw] : w.scheduled) {
            r->finished += sw;
            r->inFlight--;
        }
        if (e != cudaSuccess) {
            const int code = CudaFail(ctx_, e, "served wave");
            for (uint64_t id : std::vector<uint64_t>(active_)) Finish(*reqs_[id], PT_REQ_FAILED, code);
        } else {
            for (Request* r : w.finishing) {
                if (r->state == PT_REQ_RUNNING) Finish(*r, PT_REQ_DONE, PT_OK);
                ctx_->stats.renders++;
            }
        }
        doneCv_.notify_all();
    }

    // Two waves in flight, one per lane: once the older retires, the next is planned
    // and enqueued on its lane while the GPU runs the younger, so the GPU does not
    // wait for the host.
    void Loop() {
        cudaSetDevice(ctx_->device);
        std::deque<InFlight> flight;
        for (;;) {
            std::vector<Request*> admitted;
            std::vector<WaveUnit> units;
            InFlight w;
            int paths = 0, pixels = 0;
            {
                std::unique_lock<std::mutex> lk(mu_);
                if (flight.empty())
                    cv_.wait_for(lk, std::chrono::milliseconds(20),
                                 [&] { return stopping_ || !queue_.empty() || !active_.empty(); });
                if (stopping_) break;
                admitted = Admit();
                Plan(&units, &w, &paths, &pixels);
                doneCv_.notify_all();
            }
            if (!units.empty() || !admitted.empty()) {
                int launches = 0;
                {
                    std::lock_guard<std::mutex> cg(ctx_->mu);
                    w.error = Enqueue(admitted, units, paths, pixels, &w, &launches);
                    ctx_->stats.kernel_launches += launches;
                }
                flight.push_back(std::move(w));
            }
            if (flight.size() >= 2 || (units.empty() && !flight.empty())) Retire(flight);
        }
        while (!flight.empty()) Retire(flight);
    }

    pt_context* ctx_;
    pt_serve_config cfg_;
    std::thread thread_;
    std::mutex mu_;
    std::condition_variable cv_, doneCv_;
    bool stopping_ = false;
    std::map<uint64_t, std::unique_ptr<Request>> reqs_;
    std::deque<uint64_t> queue_;
    std::vector<uint64_t> active_;
    std::vector<int> freeSlots_;
    uint64_t nextId_ = 1;
    ArenaAllocator alloc_;
    DeviceBuffer arena_, jobTable_, units_[2], jobList_[2];  // unit tables and job lists per lane
    std::vector<DeviceBuffer> wbBufs_;
    WaveBuffers wb_[2] = {};
    int* hostCount_ = nullptr;  // pinned queue-count words of the two lanes
    WaveTuning tune_{};
    WaveGraphCache* graphs_ = nullptr;
    std::vector<DevJob> slotJobs_;
    cudaStream_t stream_[2] = {nullptr, nullptr};  // the lanes' streams
    uint64_t seq_ = 0;                              // waves enqueued (lane = seq & 1)
    // events of the latest enqueued wave while it is in flight (null once retired)
    cudaEvent_t lastSetup_ = nullptr, lastDone_ = nullptr;
    Clock::time_point t0_;
    static constexpr double kOverdueFactor = 1.0;
    static constexpr double kOverdueWaves = 6.0;
    static constexpr double kOverdueShare = 1.0;
    PathRateMeter rate_{1.5e9};  // paths per second, from the waves' retirements
};

}  // namespace ptg

using namespace ptg;

pt_context::pt_context() = default;
pt_context::~pt_context() = default;

extern "C" {

int pt_serve_start(pt_context* ctx, const pt_serve_config* config) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    pt_serve_config cfg{};
    if (config) cfg = *config;
    if (cfg.wave_paths < 0 || cfg.max_active < 0) return Fail(ctx, PT_ERR_INVALID_ARG, "bad serve config");
    std::lock_guard<std::mutex> g(ctx->mu);
    if (ctx->server) return Fail(ctx, PT_ERR_BUSY, "server already running");
    int rc = SetDevice(ctx);
    if (rc != PT_OK) return rc;
    auto s = std::make_unique<Server>(ctx, cfg);
    if ((rc = s->Start()) != PT_OK) return rc;
    ctx->server = std::move(s);
    return PT_OK;
}

int pt_serve_submit(pt_context* ctx, const pt_job* job, float* filmHost, uint64_t* id) {
    if (!ctx || !job || !id) return PT_ERR_INVALID_ARG;
    if (!ctx->server) return Fail(ctx, PT_ERR_NOT_FOUND, "server not running");
    return ctx->server->Submit(job, filmHost, id);
}

int pt_serve_poll(pt_context* ctx, uint64_t id, pt_request_status* out) {
    if (!ctx || !out) return PT_ERR_INVALID_ARG;
    if (!ctx->server) return PT_ERR_NOT_FOUND;
    return ctx->server->Poll(id, out);
}

int pt_serve_wait(pt_context* ctx, uint64_t id, double timeout, pt_request_status* out) {
    if (!ctx || !out) return PT_ERR_INVALID_ARG;
    if (!ctx->server) return PT_ERR_NOT_FOUND;
    return ctx->server->Wait(id, timeout, out);
}

int pt_serve_set_deadline(pt_context* ctx, uint64_t id, double seconds) {
    if (!ctx || !(seconds >= 0.0)) return PT_ERR_INVALID_ARG;
    if (!ctx->server) return PT_ERR_NOT_FOUND;
    return ctx->server->SetDeadline(id, seconds);
}

int pt_serve_cancel(pt_context* ctx, uint64_t id) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    if (!ctx->server) return PT_ERR_NOT_FOUND;
    return ctx->server->Cancel(id);
}

int pt_serve_release(pt_context* ctx, uint64_t id) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    if (!ctx->server) return PT_ERR_NOT_FOUND;
    return ctx->server->Release(id);
}

int pt_serve_stop(pt_context* ctx) {
    if (!ctx) return PT_ERR_INVALID_ARG;
    if (!ctx->server) return PT_ERR_NOT_FOUND;
    ctx->server->Stop();
    ctx->server.reset();
    return PT_OK;
}

}  // extern "C"
