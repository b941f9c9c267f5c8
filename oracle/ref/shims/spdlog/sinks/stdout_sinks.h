// Stand-in for the spdlog console sink named by Core/Logger.cpp (test oracle build only).
#pragma once
#include "spdlog/spdlog.h"
namespace spdlog { namespace sinks {
struct stdout_sink_mt : sink {};
} }
