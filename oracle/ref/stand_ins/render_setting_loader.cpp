// Stand-in for Core/RenderSettingLoader.cpp, whose JSON/TOML libraries are not
// available here. Reads the same keys into Petrichor::Core::RenderSetting:
//   JSON (RenderSettingLoader.cpp:49-64): outputWidth, outputHeight, spp,
//        denoising_spp, maxBounces, tileWidth, tileHeight, numThreads
//   TOML (RenderSettingLoader.cpp:105-124): settings.render_width/render_height/
//        spp/maxBounces/tile_width/tile_height/num_threads
// Only flat integer values are understood. Test oracle build only.
#include "Core/RenderSettingLoader.h"

#include <cctype>
#include <fstream>
#include <map>
#include <sstream>
#include <string>

namespace {

std::string Slurp(const std::filesystem::path& path, bool* ok) {
    std::ifstream f(path, std::ios::in | std::ios::binary);
    *ok = !f.fail();
    std::stringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

// "key": <int> pairs of a flat JSON object.
std::map<std::string, long> ParseJsonInts(const std::string& s) {
    std::map<std::string, long> out;
    size_t i = 0;
    while ((i = s.find('"', i)) != std::string::npos) {
        const size_t j = s.find('"', i + 1);
        if (j == std::string::npos) break;
        std::string key = s.substr(i + 1, j - i - 1);
        size_t k = j + 1;
        while (k < s.size() && std::isspace((unsigned char)s[k])) k++;
        if (k < s.size() && s[k] == ':') {
            k++;
            while (k < s.size() && std::isspace((unsigned char)s[k])) k++;
            size_t e = k;
            if (e < s.size() && (s[e] == '-' || s[e] == '+')) e++;
            while (e < s.size() && std::isdigit((unsigned char)s[e])) e++;
            if (e > k) out[key] = std::stol(s.substr(k, e - k));
            i = e;
        } else {
            i = j + 1;
        }
    }
    return out;
}

// "[table]" headers and "key = <int>" lines; keys are reported as "table.key".
std::map<std::string, long> ParseTomlInts(const std::string& s) {
    std::map<std::string, long> out;
    std::istringstream in(s);
    std::string line, table;
    while (std::getline(in, line)) {
        const size_t hash = line.find('#');
        if (hash != std::string::npos) line = line.substr(0, hash);
        const size_t a = line.find_first_not_of(" \t\r");
        if (a == std::string::npos) continue;
        line = line.substr(a);
        if (line[0] == '[') {
            const size_t b = line.find(']');
            table = line.substr(1, b == std::string::npos ? std::string::npos : b - 1);
            continue;
        }
        const size_t eq = line.find('=');
        if (eq == std::string::npos) continue;
        std::string key = line.substr(0, eq);
        key = key.substr(0, key.find_last_not_of(" \t") + 1);
        std::string val = line.substr(eq + 1);
        const size_t v0 = val.find_first_not_of(" \t");
        if (v0 == std::string::npos) continue;
        try {
            out[table.empty() ? key : table + "." + key] = std::stol(val.substr(v0));
        } catch (...) {
        }
    }
    return out;
}

template <typename T>
void ReadIfPresent(T* dst, const std::map<std::string, long>& kv, const char* key) {
    const auto it = kv.find(key);
    if (it != kv.end()) *dst = static_cast<T>(it->second);
}

}  // namespace

namespace Petrichor {
namespace Core {

RenderSetting RenderSettingLoaderJson::Load(const std::filesystem::path& path) {
    RenderSetting rs;
    bool ok = false;
    const auto kv = ParseJsonInts(Slurp(path, &ok));
    if (!ok) return rs;
    ReadIfPresent(&rs.outputWidth, kv, "outputWidth");
    ReadIfPresent(&rs.outputHeight, kv, "outputHeight");
    ReadIfPresent(&rs.numSamplesPerPixel, kv, "spp");
    ReadIfPresent(&rs.numSppForDenoising, kv, "denoising_spp");
    ReadIfPresent(&rs.numMaxBounces, kv, "maxBounces");
    ReadIfPresent(&rs.tileWidth, kv, "tileWidth");
    ReadIfPresent(&rs.tileHeight, kv, "tileHeight");
    ReadIfPresent(&rs.numThreads, kv, "numThreads");
    return rs;
}

RenderSetting SceneSettingsTomlLoader::Load(const std::filesystem::path& path) {
    RenderSetting rs;
    bool ok = false;
    const auto kv = ParseTomlInts(Slurp(path, &ok));
    if (!ok) return rs;
    ReadIfPresent(&rs.outputWidth, kv, "settings.render_width");
    ReadIfPresent(&rs.outputHeight, kv, "settings.render_height");
    ReadIfPresent(&rs.numSamplesPerPixel, kv, "settings.spp");
    ReadIfPresent(&rs.numMaxBounces, kv, "settings.maxBounces");
    ReadIfPresent(&rs.tileWidth, kv, "settings.tile_width");
    ReadIfPresent(&rs.tileHeight, kv, "settings.tile_height");
    ReadIfPresent(&rs.numThreads, kv, "settings.num_threads");
    return rs;
}

}  // namespace Core
}  // namespace Petrichor
