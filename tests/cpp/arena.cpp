// The serving loop's state allocator (ArenaAllocator, csrc/scheduler.h) driven without a
// device.
//
// stdin:  commands, one per line: "reset <bytes>", "alloc <bytes>", "free <offset> <bytes>"
// stdout: per alloc the offset or -1; after every command the free ranges as
//         "free <offset>:<bytes> ..." (offset order).
#include <cstdio>
#include <cstring>

#include "scheduler.h"

int main() {
    ptg::ArenaAllocator a;
    char cmd[16];
    while (std::scanf("%15s", cmd) == 1) {
        unsigned long long x = 0, y = 0;
        if (!std::strcmp(cmd, "reset")) {
            if (std::scanf("%llu", &x) != 1) return 2;
            a.Reset((size_t)x);
        } else if (!std::strcmp(cmd, "alloc")) {
            if (std::scanf("%llu", &x) != 1) return 2;
            size_t off = 0;
            if (a.Alloc((size_t)x, &off)) std::printf("at %llu\n", (unsigned long long)off);
            else std::printf("at -1\n");
        } else if (!std::strcmp(cmd, "free")) {
            if (std::scanf("%llu %llu", &x, &y) != 2) return 2;
            a.Release((size_t)x, (size_t)y);
        } else {
            return 2;
        }
        std::printf("free");
        for (const auto& [off, bytes] : a.FreeRanges())
            std::printf(" %llu:%llu", (unsigned long long)off, (unsigned long long)bytes);
        std::printf("\n");
        std::fflush(stdout);  // the caller reads each reply before it writes the next command
    }
    return 0;
}
