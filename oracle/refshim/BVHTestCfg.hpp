// Test infrastructure only: stands in for the configuration header the reference's build system
// generates from BVHTestCfg.hpp.in (version, logger name, face culling, progress bar), with the
// reference's default options and no progress output, plus the named logger accessor the
// reference's sources call.
#pragma once

#include "spdlog/spdlog.h"

namespace spd = spdlog;

#define BVHTEST_VERSION "reference-cpu-pin"
#define LOGGER_NAME "BVHTest"
#define CUDA_FACE_CULLING 1
#define ENABLE_PROGRESS_BAR 0

namespace BVHTest {

inline auto getLogger() {
  auto lLogger = spd::get(LOGGER_NAME);
  if (!lLogger) lLogger = spd::stdout_color_mt(LOGGER_NAME);
  return lLogger;
}

}  // namespace BVHTest
