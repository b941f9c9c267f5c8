// Host-side wave scheduling for the wavefront kernels: splits each job into
// sample blocks (work units over all of its pixels), packs units into waves of at
// most `waveCapacity` paths, runs the waves in order and finalizes each job after
// its last wave. A job's sample blocks are visited in increasing sample order, so
// its per-pixel sums (and its film) are the same in any packing. Also the serving
// loop's host parts that need no device: its wave plan, its state allocator and its
// path-rate meter.
#pragma once
#include <stddef.h>

#include <iterator>
#include <map>
#include <utility>
#include <vector>

#include "pt_kernels.h"

namespace ptg {

struct WaveTables {      // device buffers owned by the caller
    DevJob* jobs;        // >= number of jobs
    WaveUnit* units;     // >= maxUnits
    WaveUnit* units2;    // >= maxUnits: the second wave lane's units (may be null: one lane)
    int* jobList;        // >= number of jobs
    int maxUnits;
};

// Plans the waves for `jobs` (spp, width, height taken from each job's settings).
// Returns false when one sample of some job does not fit in a wave.
bool PlanWaves(const std::vector<DevJob>& jobs, int waveCapacity, int maxUnits,
               std::vector<std::vector<WaveUnit>>* waves);

// Renders the jobs: uploads the job table, zeroes each job's sums, runs every
// wave and finalizes jobs as they complete. Enqueued on `stream` (synchronises
// only for SimplePathTracing queue polls).
cudaError_t RenderJobs(const std::vector<DevJob>& jobs, const WaveTables& tables,
                       const WaveBuffers& wb, int waveCapacity, cudaStream_t stream, int* launches,
                       WaveProfile* prof, const WaveTuning& tune = WaveTuning{},
                       WaveGraphCache* graphs = nullptr);

// Bounce iterations a wave needs: maxBounces + 1 for PathTracing jobs; -1 (run
// until the queue drains) when a SimplePathTracing job is present.
int WaveIterations(const std::vector<DevJob>& jobs, const std::vector<WaveUnit>& units);
// The integrator shared by all of a wave's jobs, or -1 when they differ.
int WaveIntegrator(const std::vector<DevJob>& jobs, const std::vector<WaveUnit>& units);
// The job of all of a wave's units, or -1 when they belong to several.
int WaveSoleJob(const std::vector<WaveUnit>& units);
// 1 when a job of the wave has area lights (its next-event rays include closest-hit ones).
int WaveAreaLights(const std::vector<DevJob>& jobs, const std::vector<WaveUnit>& units);
// The shape of a wave of these units (path and pixel counts, iterations, integrator,
// sole job, area lights, rasterised units, which it moves last and renumbers).
WaveShape ShapeOf(const std::vector<DevJob>& jobs, std::vector<WaveUnit>& units,
                  int primaryTraversal);
// Rays per triangle from which a unit's first bounce is rasterised by default. Measured
// on GB300 with films alike: at 133 (1.0M triangles, 1920x1080, 64 spp) the raster pass
// takes 5.5 ms against about 10 ms of first-bounce traversal; at 3.3 (20.0M triangles,
// 3840x2160, waves of 8 spp) it takes 21 ms per wave against 13 ms, its per-triangle work
// (one warp visit per row segment) outweighing the rays it saves.
constexpr int64_t kRasterMinPathsPerTri = 16;
// Picks the units whose first bounce is rasterised (a pinhole PathTracing job with at
// least kRasterMinPathsPerTri of the unit's rays per triangle, or 2 with
// primaryTraversal 2; none with primaryTraversal 1 or in a queue-polled wave), moves
// them after the traced units, renumbers every unit's path and pixel ranges, gives each
// its record base, and sets shape's raster, rasterFrom and rasterUnit0 (shape's nPaths
// and iters already set). A wave's films do not depend on its unit order.
void PrepareRasterUnits(const std::vector<DevJob>& jobs, std::vector<WaveUnit>* units,
                        WaveShape* shape, int primaryTraversal);

// ---- the serving loop's wave plan (server.cpp)
// A request that still has samples to plan: its pixels, samples, samples already planned
// and submission time (seconds).
struct ServeRequestView {
    int pixels, spp, scheduled;
    double submit;
};
struct ServePlanLimits {
    int cap;                   // paths per wave
    int maxUnits;              // sample blocks per wave
    double now;                // seconds, on the submission clock
    double pathRate;           // paths per second (measured)
    double overdueWaves;       // a request is overdue after this many waves' time ...
    double overdueFactor;      // ... plus this many times its own rendering time
    double overdueShare;       // share of every wave guaranteed to overdue requests
};
// One sample block of the next wave: the request (index into the views) and its samples;
// blocks are listed in the wave's path order.
struct ServePick {
    int request, sw;
};
// Packs the next wave, least remaining work first (a short request finishes in the next
// wave; long ones take what is left). Under sustained load that order would keep
// postponing the longest requests, so a request is overdue once it has waited
// overdueWaves waves (cap / pathRate each) plus overdueFactor times its own rendering
// time (spp * pixels / pathRate), and the overdue ones, oldest first, are guaranteed
// overdueShare of the wave (as much of it as they can use). Each request gets at most
// one block per wave.
std::vector<ServePick> PlanServeWave(const std::vector<ServeRequestView>& reqs,
                                     const ServePlanLimits& lim);

// First-fit allocator over the offsets of one device buffer, in 256-byte granules: the
// serving loop's per-request state (sums, film staging) within its state budget. Released
// ranges merge with free neighbours.
class ArenaAllocator {
public:
    void Reset(size_t bytes) {
        free_.clear();
        if (bytes) free_[0] = bytes;
    }
    // The lowest free offset with room for `bytes` (rounded up to 256); false if none.
    bool Alloc(size_t bytes, size_t* off) {
        bytes = (bytes + 255) & ~size_t(255);
        for (auto it = free_.begin(); it != free_.end(); ++it) {
            if (it->second >= bytes) {
                *off = it->first;
                const size_t rest = it->second - bytes, start = it->first + bytes;
                free_.erase(it);
                if (rest) free_[start] = rest;
                return true;
            }
        }
        return false;
    }
    // Returns a range Alloc gave (the same `bytes`).
    void Release(size_t off, size_t bytes) {
        bytes = (bytes + 255) & ~size_t(255);
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
    const std::map<size_t, size_t>& FreeRanges() const { return free_; }  // offset -> bytes

private:
    std::map<size_t, size_t> free_;
};

// The GPU's path rate, from wave retirements: the paths retired over the span of the last
// kWindow gaps between retirements of one busy period (another wave in flight at each),
// smoothed. Two waves run at once on the serving loop's two lanes, so consecutive
// retirements can fall close together; single gaps would overstate the rate and make every
// request look overdue. A retirement after which no wave is in flight ends the busy period:
// the GPU may idle before the next wave, so the next retirement starts a new window.
class PathRateMeter {
public:
    static constexpr int kWindow = 4;
    explicit PathRateMeter(double initial) : rate_(initial) {}
    // A wave of `paths` retired at `now` (seconds); ok: it ran without error; busyAfter:
    // another wave is still in flight.
    void Retired(double now, int64_t paths, bool ok, bool busyAfter);
    double Rate() const { return rate_; }

private:
    double rate_;
    bool busy_ = false;                              // the previous retirement left a wave in flight
    std::vector<std::pair<double, int64_t>> recent_;  // (time, paths), oldest first
};

}  // namespace ptg
