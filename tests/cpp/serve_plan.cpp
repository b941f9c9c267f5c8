// The serving loop's wave plan (PlanServeWave, csrc/scheduler.h) driven without a device.
//
// stdin:  nQueries, then per query
//           cap maxUnits now pathRate overdueWaves overdueFactor overdueShare nRequests
//           and per request: pixels spp scheduled submit
// stdout: per query a line "plan <k>" followed by one line per block "pick <request> <sw>",
//         in the wave's path order.
#include <cstdio>
#include <vector>

#include "scheduler.h"

int main() {
    int q = 0;
    if (std::scanf("%d", &q) != 1 || q < 0) return 2;
    for (int k = 0; k < q; k++) {
        ptg::ServePlanLimits lim{};
        int n = 0;
        if (std::scanf("%d %d %lf %lf %lf %lf %lf %d", &lim.cap, &lim.maxUnits, &lim.now, &lim.pathRate,
                       &lim.overdueWaves, &lim.overdueFactor, &lim.overdueShare, &n) != 8 || n < 0)
            return 2;
        std::vector<ptg::ServeRequestView> reqs(n);
        for (ptg::ServeRequestView& r : reqs)
            if (std::scanf("%d %d %d %lf", &r.pixels, &r.spp, &r.scheduled, &r.submit) != 4 || r.pixels < 1)
                return 2;
        std::printf("plan %d\n", k);
        for (const ptg::ServePick& p : ptg::PlanServeWave(reqs, lim))
            std::printf("pick %d %d\n", p.request, p.sw);
    }
    return 0;
}
