// The serving loop's path-rate meter (PathRateMeter, csrc/scheduler.h) driven without a
// device.
//
// stdin:  initialRate, then one retirement per line: now paths ok busyAfter
// stdout: the meter's rate after each retirement, one per line.
#include <cstdio>

#include "scheduler.h"

int main() {
    double initial = 0.0;
    if (std::scanf("%lf", &initial) != 1) return 2;
    ptg::PathRateMeter meter(initial);
    double now = 0.0;
    long long paths = 0;
    int ok = 0, busy = 0;
    while (std::scanf("%lf %lld %d %d", &now, &paths, &ok, &busy) == 4) {
        meter.Retired(now, paths, ok != 0, busy != 0);
        std::printf("%.9g\n", meter.Rate());
    }
    return 0;
}
