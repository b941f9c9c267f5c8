// Stand-in for the spdlog file sink named by Core/Logger.cpp (test oracle build only).
#pragma once
#include <string>
#include "spdlog/spdlog.h"
namespace spdlog { namespace sinks {
struct basic_file_sink_mt : sink {
    explicit basic_file_sink_mt(const std::string&) {}
};
} }
