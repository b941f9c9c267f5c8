// Wave scheduling for the wavefront kernels (see scheduler.h).
#include "scheduler.h"

#include <algorithm>
#include <cmath>

namespace ptg {

void* NewStageEvents();

bool PlanWaves(const std::vector<DevJob>& jobs, int cap, int maxUnits,
               std::vector<std::vector<WaveUnit>>* waves) {
    waves->clear();
    std::vector<WaveUnit> cur;
    int curPaths = 0, curPixels = 0;
    auto flush = [&]() {
        if (!cur.empty()) waves->push_back(cur);
        cur.clear();
        curPaths = curPixels = 0;
    };
    for (size_t j = 0; j < jobs.size(); j++) {
        const int P = jobs[j].st.width * jobs[j].st.height;
        const int spp = jobs[j].st.spp;
        if (P > cap) return false;
        for (int s0 = 0; s0 < spp;) {
            int room = (cap - curPaths) / P;
            if (room < 1 || (int)cur.size() >= maxUnits) {
                flush();
                room = cap / P;
            }
            const int sw = std::min(spp - s0, room);
            WaveUnit u{};
            u.job = (int)j;
            u.s0 = s0;
            u.sw = sw;
            u.pathBase = curPaths;
            u.pixelBase = curPixels;
            cur.push_back(u);
            curPaths += P * sw;
            curPixels += P;
            s0 += sw;
        }
    }
    flush();
    return true;
}

int WaveIterations(const std::vector<DevJob>& jobs, const std::vector<WaveUnit>& units) {
    int iters = 0;
    for (const WaveUnit& u : units) {
        const DevSettings& st = jobs[u.job].st;
        if (st.integrator == kSimplePathTracing) return -1;
        iters = std::max(iters, st.maxBounces + 1);
    }
    return iters;
}

int WaveIntegrator(const std::vector<DevJob>& jobs, const std::vector<WaveUnit>& units) {
    int integ = -2;
    for (const WaveUnit& u : units) {
        const int k = jobs[u.job].st.integrator;
        if (integ == -2) integ = k;
        else if (integ != k) return -1;
    }
    return integ < 0 ? -1 : integ;
}

void PrepareRasterUnits(const std::vector<DevJob>& jobs, std::vector<WaveUnit>* units,
                        WaveShape* shape, int primaryTraversal) {
    shape->raster = 0;
    shape->rasterFrom = shape->nPaths;
    shape->rasterUnit0 = (int)units->size();
    if (primaryTraversal == 1) {  // every first bounce traced
        for (WaveUnit& u : *units) u.recBase = -1;
        return;
    }
    // rays per triangle: at least kRasterMinPathsPerTri to pick rasterisation by itself;
    // at least 2 in any case, which keeps the per-triangle records (64 B each) within half
    // of the shadow queue (64 B per path) the raster kernels carve them from
    const int64_t perTri = primaryTraversal == 2 ? 2 : kRasterMinPathsPerTri;
    std::vector<WaveUnit> trace, raster;
    for (WaveUnit u : *units) {
        const DevJob& J = jobs[u.job];
        const int64_t paths = (int64_t)J.st.width * J.st.height * u.sw;
        // a camera within twice the scene's largest coordinate of the origin: then a hit
        // point inside its triangle's bounds is certainly inside its leaf box by a margin
        // (raster_primary.cuh HitNearTriangle) of at least a quarter of the box widening
        const float camMax = std::max(std::fabs(J.C.pos[0]), std::max(std::fabs(J.C.pos[1]),
                                                                      std::fabs(J.C.pos[2])));
        const bool near = camMax <= 2.0f * std::ldexp(J.S.wideEps, 18);
        const bool ok = shape->iters >= 0 && J.C.aperture == 0.0f && J.S.numTris > 0 && near &&
                        J.st.width < 65536 && J.st.height < 65536 &&
                        J.st.integrator == kPathTracing &&
                        paths >= perTri * (int64_t)J.S.numTris &&
                        (int64_t)shape->raster + J.S.numTris < (int64_t(1) << 30);
        u.recBase = -1;
        if (ok) {
            u.recBase = shape->raster;
            shape->raster += J.S.numTris;
            raster.push_back(u);
        } else {
            trace.push_back(u);
        }
    }
    if (raster.empty()) {
        for (WaveUnit& u : *units) u.recBase = -1;
        return;
    }
    // traced units first, rasterised units last; path and pixel ranges follow the order
    units->clear();
    units->insert(units->end(), trace.begin(), trace.end());
    units->insert(units->end(), raster.begin(), raster.end());
    int paths = 0, pixels = 0;
    for (size_t k = 0; k < units->size(); k++) {
        WaveUnit& u = (*units)[k];
        const int P = jobs[u.job].st.width * jobs[u.job].st.height;
        if (k == trace.size()) shape->rasterFrom = paths;
        u.pathBase = paths;
        u.pixelBase = pixels;
        paths += P * u.sw;
        pixels += P;
    }
    shape->rasterUnit0 = (int)trace.size();
}

std::vector<ServePick> PlanServeWave(const std::vector<ServeRequestView>& reqs,
                                     const ServePlanLimits& lim) {
    const double slack = lim.overdueWaves * lim.cap / lim.pathRate;
    std::vector<int> fresh, overdue;
    int64_t overdueWork = 0;
    for (int i = 0; i < (int)reqs.size(); i++) {
        const ServeRequestView& r = reqs[i];
        if (r.scheduled >= r.spp) continue;
        const double own = (double)r.spp * r.pixels / lim.pathRate;
        if (lim.now - r.submit > slack + lim.overdueFactor * own) {
            overdue.push_back(i);
            overdueWork += (int64_t)(r.spp - r.scheduled) * r.pixels;
        } else {
            fresh.push_back(i);
        }
    }
    auto remaining = [&](int i) { return (int64_t)(reqs[i].spp - reqs[i].scheduled) * reqs[i].pixels; };
    std::stable_sort(fresh.begin(), fresh.end(), [&](int a, int b) { return remaining(a) < remaining(b); });
    std::stable_sort(overdue.begin(), overdue.end(),
                     [&](int a, int b) { return reqs[a].submit < reqs[b].submit; });
    const int reserve = (int)std::min<int64_t>((int64_t)(lim.overdueShare * lim.cap), overdueWork);
    std::vector<ServePick> picks;
    int paths = 0;
    auto place = [&](int i, int limit) {
        const ServeRequestView& r = reqs[i];
        const int room = (limit - paths) / r.pixels;
        if (room < 1 || (int)picks.size() >= lim.maxUnits) return false;
        const int sw = std::min(r.spp - r.scheduled, room);
        picks.push_back({i, sw});
        paths += r.pixels * sw;
        return true;
    };
    std::vector<char> placed(fresh.size(), 0);
    for (size_t k = 0; k < fresh.size(); k++) placed[k] = place(fresh[k], lim.cap - reserve);
    for (int i : overdue) place(i, lim.cap);
    for (size_t k = 0; k < fresh.size(); k++)
        if (!placed[k]) place(fresh[k], lim.cap);
    return picks;
}

void PathRateMeter::Retired(double now, int64_t paths, bool ok, bool busyAfter) {
    if (ok) {
        if (!busy_) recent_.clear();
        recent_.push_back({now, paths});
        if ((int)recent_.size() > kWindow + 1) recent_.erase(recent_.begin());
        int64_t sum = 0;
        for (size_t i = 1; i < recent_.size(); i++) sum += recent_[i].second;
        const double span = recent_.back().first - recent_.front().first;
        if ((int)recent_.size() == kWindow + 1 && span > 0.0 && sum > (int64_t)1 << 20)
            rate_ = 0.75 * rate_ + 0.25 * ((double)sum / span);
    }
    busy_ = busyAfter;
}

int WaveAreaLights(const std::vector<DevJob>& jobs, const std::vector<WaveUnit>& units) {
    for (const WaveUnit& u : units)
        if (jobs[u.job].S.numLights > 0) return 1;
    return 0;
}

int WaveSoleJob(const std::vector<WaveUnit>& units) {
    for (const WaveUnit& u : units)
        if (u.job != units.front().job) return -1;
    return units.empty() ? -1 : units.front().job;
}

WaveShape ShapeOf(const std::vector<DevJob>& jobs, std::vector<WaveUnit>& units,
                  int primaryTraversal) {
    WaveShape shape;
    for (const WaveUnit& u : units) {
        const int P = jobs[u.job].st.width * jobs[u.job].st.height;
        shape.nPaths += P * u.sw;
        shape.nPixelUnits += P;
    }
    shape.nUnits = (int)units.size();
    shape.iters = WaveIterations(jobs, units);
    shape.integrator = WaveIntegrator(jobs, units);
    shape.soleJob = WaveSoleJob(units);
    shape.areaLights = WaveAreaLights(jobs, units);
    PrepareRasterUnits(jobs, &units, &shape, primaryTraversal);
    return shape;
}

namespace {

// Finalises the jobs whose last wave is w (film = sums / spp), on `stream`.
cudaError_t FinalizeDone(const std::vector<DevJob>& jobs, const WaveTables& T,
                         const std::vector<int>& lastWave, size_t w, cudaStream_t stream,
                         int* launches, WaveProfile* prof) {
    std::vector<int> done;
    int maxPx = 0;
    for (size_t j = 0; j < jobs.size(); j++)
        if (lastWave[j] == (int)w) {
            done.push_back((int)j);
            maxPx = std::max(maxPx, jobs[j].st.width * jobs[j].st.height);
        }
    if (done.empty()) return cudaSuccess;
    cudaError_t e = cudaMemcpyAsync(T.jobList, done.data(), done.size() * sizeof(int),
                                    cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    return FinalizeJobs(T.jobs, T.jobList, (int)done.size(), maxPx, stream, launches, prof);
}

}  // namespace

// Waves run one after another on `stream`, or, when a render needs more than one wave
// and the buffers hold two half-size sets, on two streams in turn: wave w+1 starts
// while wave w finishes its last, sparse bounces, so the late-bounce tail of every wave
// but the last is hidden. Each wave accumulates only after the previous wave has
// accumulated and finalised (an event chain), so pixels still sum their samples in
// sample order and films do not depend on the lane schedule.
cudaError_t RenderJobs(const std::vector<DevJob>& jobs, const WaveTables& T, const WaveBuffers& wb,
                       int cap, cudaStream_t stream, int* launches, WaveProfile* prof,
                       const WaveTuning& tune, WaveGraphCache* graphs) {
    std::vector<std::vector<WaveUnit>> waves;
    if (!PlanWaves(jobs, std::min(cap, wb.capacity), T.maxUnits, &waves))
        return cudaErrorInvalidValue;
    // two lanes: half-capacity sets carved from the same allocation
    WaveBuffers lane[2];
    cudaStream_t laneStream[2] = {stream, nullptr};
    cudaEvent_t done[2] = {nullptr, nullptr};
    bool twoLanes = false;
    if (waves.size() > 1 && !prof && graphs && T.units2 && wb.bytes > 0 &&
        wb.bytes >= 2 * WaveBuffersBytes(wb.capacity / 2) &&
        WavePipeline(graphs, &laneStream[1], done)) {
        std::vector<std::vector<WaveUnit>> half;
        if (PlanWaves(jobs, std::min(cap, wb.capacity) / 2, T.maxUnits, &half)) {
            char* base = reinterpret_cast<char*>(wb.ray[0]);
            lane[0] = CarveWaveBuffers(base, wb.capacity / 2);
            lane[1] = CarveWaveBuffers(base + WaveBuffersBytes(wb.capacity / 2), wb.capacity / 2);
            lane[0].hostCount = wb.hostCount;
            lane[1].hostCount = wb.hostCount ? wb.hostCount + 1 : nullptr;
            waves.swap(half);
            twoLanes = true;
        }
    }
    cudaError_t e = cudaMemcpyAsync(T.jobs, jobs.data(), jobs.size() * sizeof(DevJob),
                                    cudaMemcpyHostToDevice, stream);
    if (e != cudaSuccess) return e;
    for (const DevJob& J : jobs) {
        e = cudaMemsetAsync(J.accum, 0, sizeof(float4) * (size_t)J.st.width * J.st.height, stream);
        if (e != cudaSuccess) return e;
    }
    if (prof && !prof->events) prof->events = NewStageEvents();
    std::vector<int> lastWave(jobs.size(), -1);
    for (size_t w = 0; w < waves.size(); w++)
        for (const WaveUnit& u : waves[w]) lastWave[u.job] = (int)w;
    if (!twoLanes) {
        e = cudaMemsetAsync(wb.counts, 0, 16 * sizeof(int), stream);
        for (size_t w = 0; w < waves.size() && e == cudaSuccess; w++) {
            std::vector<WaveUnit>& units = waves[w];
            const WaveShape shape = ShapeOf(jobs, units, tune.primaryTraversal);  // may reorder the units
            // pageable source: the copy is staged before the call returns, so the
            // next wave may reuse the host vector
            e = cudaMemcpyAsync(T.units, units.data(), units.size() * sizeof(WaveUnit),
                                cudaMemcpyHostToDevice, stream);
            if (e == cudaSuccess)
                e = RunWave(T.jobs, T.units, shape, wb, stream, launches, prof, tune, graphs);
            if (e == cudaSuccess) e = FinalizeDone(jobs, T, lastWave, w, stream, launches, prof);
        }
        return e;
    }
    // the side lane starts after the job table, sums and counters are in place
    for (int k = 0; k < 2 && e == cudaSuccess; k++)
        e = cudaMemsetAsync(lane[k].counts, 0, 16 * sizeof(int), stream);
    if (e == cudaSuccess) e = cudaEventRecord(done[1], stream);
    if (e == cudaSuccess) e = cudaStreamWaitEvent(laneStream[1], done[1], 0);
    WaveUnit* unitTable[2] = {T.units, T.units2};
    for (size_t w = 0; w < waves.size() && e == cudaSuccess; w++) {
        const int k = (int)(w & 1);
        cudaStream_t s = laneStream[k];
        std::vector<WaveUnit>& units = waves[w];
        const WaveShape shape = ShapeOf(jobs, units, tune.primaryTraversal);  // may reorder the units
        e = cudaMemcpyAsync(unitTable[k], units.data(), units.size() * sizeof(WaveUnit),
                            cudaMemcpyHostToDevice, s);
        if (e == cudaSuccess)
            e = RunWave(T.jobs, unitTable[k], shape, lane[k], s, launches, nullptr, tune, graphs, k,
                        false);
        // accumulate and finalise after the previous wave did
        if (e == cudaSuccess && w > 0) e = cudaStreamWaitEvent(s, done[k ^ 1], 0);
        if (e == cudaSuccess) e = AccumulateWave(T.jobs, unitTable[k], lane[k], tune, s, launches);
        if (e == cudaSuccess) e = FinalizeDone(jobs, T, lastWave, w, s, launches, nullptr);
        if (e == cudaSuccess) e = cudaEventRecord(done[k], s);
    }
    // the caller's stream continues after the last wave (whose chain covers every wave)
    if (e == cudaSuccess) e = cudaStreamWaitEvent(stream, done[(waves.size() - 1) & 1], 0);
    if (e == cudaSuccess) e = MergeWaveErrors(wb, lane[0], lane[1], stream);
    return e;
}

}  // namespace ptg
