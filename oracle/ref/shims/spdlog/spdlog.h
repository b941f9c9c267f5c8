// Minimal logging stand-in with the spdlog names the reference's Logger uses
// (Core/Logger.h: logger::info/error, logger::sinks()). Written for building the
// reference as a test oracle only; messages are dropped unless PT_REF_VERBOSE is set.
#pragma once
#include <cstdio>
#include <cstdlib>
#include <memory>
#include <string>
#include <string_view>
#include <type_traits>
#include <vector>

namespace spdlog {
namespace sinks {
struct sink {
    virtual ~sink() = default;
};
}  // namespace sinks

class logger {
public:
    explicit logger(std::string name) : m_name(std::move(name)) {}
    template <typename T, typename... A>
    void info(const T& first, const A&...) { emit("info", first); }
    template <typename T, typename... A>
    void error(const T& first, const A&...) { emit("error", first); }
    std::vector<std::shared_ptr<sinks::sink>>& sinks() { return m_sinks; }

private:
    template <typename T>
    void emit(const char* level, const T& first) {
        if (!std::getenv("PT_REF_VERBOSE")) return;
        if constexpr (std::is_convertible_v<T, std::string_view>) {
            std::string_view s(first);
            std::fprintf(stderr, "[%s] %.*s\n", level, (int)s.size(), s.data());
        } else {
            std::fprintf(stderr, "[%s] (object)\n", level);
        }
    }
    std::string m_name;
    std::vector<std::shared_ptr<sinks::sink>> m_sinks;
};
}  // namespace spdlog
