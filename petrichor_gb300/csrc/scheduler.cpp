// Wave scheduling for the wavefront kernels (see scheduler.h).
#include "scheduler.h"

#include <algorithm>

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

int WaveSoleJob(const std::vector<WaveUnit>& units) {
    for (const WaveUnit& u : units)
        if (u.job != units.front().job) return -1;
    return units.empty() ? -1 : units.front().job;
}

cudaError_t RenderJobs(const std::vector<DevJob>& jobs, const WaveTables& T, const WaveBuffers& wb,
                       int cap, cudaStream_t stream, int* launches, WaveProfile* prof,
                       const WaveTuning& tune, WaveGraphCache* graphs) {
    std::vector<std::vector<WaveUnit>> waves;
    if (!PlanWaves(jobs, std::min(cap, wb.capacity), T.maxUnits, &waves))
        return cudaErrorInvalidValue;
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
    for (size_t w = 0; w < waves.size(); w++) {
        const std::vector<WaveUnit>& units = waves[w];
        // pageable source: the copy is staged before the call returns, so the
        // next wave may reuse the host vector
        e = cudaMemcpyAsync(T.units, units.data(), units.size() * sizeof(WaveUnit),
                            cudaMemcpyHostToDevice, stream);
        if (e != cudaSuccess) return e;
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
        e = RunWave(T.jobs, T.units, shape, wb, stream, launches, prof, tune, graphs);
        if (e != cudaSuccess) return e;
        std::vector<int> done;
        int maxPx = 0;
        for (size_t j = 0; j < jobs.size(); j++)
            if (lastWave[j] == (int)w) {
                done.push_back((int)j);
                maxPx = std::max(maxPx, jobs[j].st.width * jobs[j].st.height);
            }
        if (!done.empty()) {
            e = cudaMemcpyAsync(T.jobList, done.data(), done.size() * sizeof(int),
                                cudaMemcpyHostToDevice, stream);
            if (e != cudaSuccess) return e;
            e = FinalizeJobs(T.jobs, T.jobList, (int)done.size(), maxPx, stream, launches, prof);
            if (e != cudaSuccess) return e;
        }
    }
    return cudaSuccess;
}

}  // namespace ptg
