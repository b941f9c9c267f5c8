// Adversarial input for std::sort (M. D. McIlroy, "A killer adversary for quicksort",
// Software: Practice and Experience 29(4), 1999): std::sort runs on indices with a
// comparator that fixes values lazily ("gas" until compared), freezing the element
// the partition step is most likely to use as pivot. The values it ends with make
// the same std::sort take the same bad partitions, so introsort exhausts its depth
// budget and falls back to heapsort.
//
//   antiqsort <n>   prints n integer keys, one per line
#include <algorithm>
#include <cstdio>
#include <cstdlib>
#include <numeric>
#include <vector>

namespace {
std::vector<int> val;
int gas = 0, nsolid = 0, candidate = 0;

struct Adversary {
    bool operator()(int x, int y) const {
        if (val[x] == gas && val[y] == gas) val[x == candidate ? x : y] = nsolid++;
        if (val[x] == gas) candidate = x;
        else if (val[y] == gas) candidate = y;
        return val[x] < val[y];
    }
};
}  // namespace

int main(int argc, char** argv) {
    if (argc < 2) return 2;
    const int n = std::atoi(argv[1]);
    if (n <= 0) return 2;
    gas = n;
    val.assign(n, gas);
    std::vector<int> ptr(n);
    std::iota(ptr.begin(), ptr.end(), 0);
    std::sort(ptr.begin(), ptr.end(), Adversary());
    for (int i = 0; i < n; i++) std::printf("%d\n", val[i]);
    return 0;
}
