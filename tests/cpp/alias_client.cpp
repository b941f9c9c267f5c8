// The alias-method test of the reference (TestPetrichor/Math/TestAliasMethod.cpp:16-94)
// run against Petrichor::Math::AliasMethod of the C++ API: random 10-bin integer
// distributions, samples drawn with two Marsaglia xor128 streams (seeds 13241 and
// 51234, next() = u32 / 2^32), and per distribution the reference's statistic
// sum (p - f)^2 / p on normalised frequencies plus a count-based chi-square.
//
//   alias_client <distributions> <samples>   prints "max_stat max_chi2"
#include <petrichor_gb300/Petrichor.hpp>

#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <random>
#include <vector>

namespace {
struct Xor128 {  // Marsaglia xor128 with the reference's initial state (Random/XorShift.h)
    uint32_t x = 123456789, y = 362436069, z = 521288629, w;
    explicit Xor128(uint32_t seed) : w(seed) {}
    float Next() {
        const uint32_t t = x ^ (x << 11);
        x = y;
        y = z;
        z = w;
        w = (w ^ (w >> 19)) ^ (t ^ (t >> 8));
        return static_cast<float>(w) / 4294967296.0f;
    }
};
}  // namespace

int main(int argc, char** argv) {
    if (argc < 3) return 2;
    const int tests = std::atoi(argv[1]), samples = std::atoi(argv[2]);
    std::mt19937 rng(36917234);
    std::uniform_int_distribution<> uniformInt(0, 1000000);
    double maxStat = 0.0, maxChi2 = 0.0;
    for (int t = 0; t < tests; t++) {
        std::vector<int> input(10);
        double sum = 0.0;
        for (int& v : input) sum += (v = uniformInt(rng));
        Petrichor::Math::AliasMethod alias;
        alias.Construct(input);
        Xor128 r0(13241), r1(51234);
        std::vector<double> freq(10, 0.0);
        for (int i = 0; i < samples; i++) {
            float a = r0.Next(), b = r1.Next();
            if (a >= 1.0f) a = 0.99999994f;  // u32 / 2^32 rounds to 1 for the largest values
            if (b >= 1.0f) b = 0.99999994f;
            freq[alias.Sample(a, b)] += 1.0;
        }
        double stat = 0.0, chi2 = 0.0;
        for (int k = 0; k < 10; k++) {
            const double p = input[k] / sum, f = freq[k] / samples;
            if (p == 0.0) continue;
            stat += (p - f) * (p - f) / p;
            const double e = p * samples;
            chi2 += (freq[k] - e) * (freq[k] - e) / e;
        }
        maxStat = stat > maxStat ? stat : maxStat;
        maxChi2 = chi2 > maxChi2 ? chi2 : maxChi2;
    }
    std::printf("%.6g %.6g\n", maxStat, maxChi2);
    return 0;
}
