// Host-side wave planning (csrc/scheduler.h) driven without a device: reads a job list,
// plans its waves with PlanWaves and shapes each one with ShapeOf (the first-bounce
// rasterisation choice, which reorders and renumbers the units), and prints every wave.
//
// stdin:  cap maxUnits primaryTraversal nJobs
//         then per job: width height spp maxBounces integrator aperture numTris camX wideEps
// stdout: "plan failed" when PlanWaves refuses the jobs; otherwise per wave a line
//         "wave nPaths nPixelUnits iters integrator soleJob raster rasterFrom rasterUnit0 nUnits"
//         followed by one line per unit "unit job s0 sw pathBase pixelBase recBase".
#include <cstdio>
#include <vector>

#include "scheduler.h"

int main() {
    int cap = 0, maxUnits = 0, primary = 0, n = 0;
    if (std::scanf("%d %d %d %d", &cap, &maxUnits, &primary, &n) != 4 || n < 0) return 2;
    std::vector<ptg::DevJob> jobs(n);
    for (ptg::DevJob& J : jobs) {
        J = ptg::DevJob{};
        float aperture = 0.0f, camX = 0.0f, eps = 0.0f;
        if (std::scanf("%d %d %d %d %d %f %d %f %f", &J.st.width, &J.st.height, &J.st.spp,
                       &J.st.maxBounces, &J.st.integrator, &aperture, &J.S.numTris, &camX, &eps) != 9)
            return 2;
        J.C.aperture = aperture;
        J.C.pos[0] = camX;
        J.S.wideEps = eps;
    }
    std::vector<std::vector<ptg::WaveUnit>> waves;
    if (!ptg::PlanWaves(jobs, cap, maxUnits, &waves)) {
        std::printf("plan failed\n");
        return 0;
    }
    for (std::vector<ptg::WaveUnit>& units : waves) {
        const ptg::WaveShape s = ptg::ShapeOf(jobs, units, primary);
        std::printf("wave %d %d %d %d %d %d %d %d %d\n", s.nPaths, s.nPixelUnits, s.iters, s.integrator,
                    s.soleJob, s.raster, s.rasterFrom, s.rasterUnit0, s.nUnits);
        for (const ptg::WaveUnit& u : units)
            std::printf("unit %d %d %d %d %d %d\n", u.job, u.s0, u.sw, u.pathBase, u.pixelBase, u.recBase);
    }
    return 0;
}
