// BVHTest's command/state framework over the C ABI: the commands keep the reference's names,
// JSON option keys and defaults, requirement bits and error codes, so existing config files run
// unchanged (lib/base/Command.*, State.hpp, Config.*, src/main.cpp).
#pragma once

#include <chrono>
#include <cstdint>
#include <memory>
#include <string>
#include <vector>

#include "../../include/bvhgb.h"
#include "json.hpp"

namespace bvhgb::host {

// ErrorCode (lib/base/Command.hpp:33-42).
enum class ErrorCode : int { OK = 0, WARNING, IO_ERROR, PARSE_ERROR, BVH_ERROR, GL_ERROR, CUDA_ERROR, GENERIC_ERROR };
const char *to_string(ErrorCode e);
ErrorCode from_status(int status);  // bvhgb_status -> ErrorCode

// CommandType (lib/base/State.hpp:32-43).
enum CommandType : uint64_t {
  IMPORT = 1ull << 0,
  BVH_BUILD = 1ull << 4,
  BVH_OPT1 = 1ull << 5,
  BVH_OPT2 = 1ull << 6,
  CUDA_DONE = 1ull << 7,
  CUDA_INIT = 1ull << 8,
  RAY_TRACE = 1ull << 16,
  EXPORT = 1ull << 24,
  SUMMARY = 1ull << 28,
};

struct CameraDesc {  // Camera::CAMERA + RES (lib/misc/Camera.hpp:27-32, CameraBase.hpp:28-31)
  float pos[3] = {0.0f, 0.0f, 2.0f};
  float lookAt[3] = {0.0f, 0.0f, 0.0f};
  float up[3] = {0.0f, 1.0f, 0.0f};
  float fov = 45.0f;
  uint32_t width = 2560, height = 1440;
  void fromJSON(const Json &j);
  Json toJSON() const;
};

// State (lib/base/State.hpp:46-99).
struct State {
  uint64_t commandsRun = 0;
  std::string basePath, input, name;
  struct CMD {
    std::string name;
    uint64_t type;
    double ms;
  };
  std::vector<CMD> commands;
  struct OptStep {
    uint32_t step;
    float sah;
    double ms;
  };
  struct {
    std::vector<OptStep> optStepps;
    uint64_t numSkipped = 0, numTotal = 0;
  } optData;
  // host mesh (Mesh) and BVH
  std::vector<float> vert, norm;
  std::vector<uint32_t> faces;
  std::vector<bvhgb_node> bvh;
  uint32_t root = 0;
  uint16_t maxLevel = 0;
  // device memory (CudaMemory)
  bvhgb_mesh_raw rawMesh{};
  bvhgb_bvh_pointer cudaBVH{};
  std::vector<CameraDesc> cameras;
  struct Work {
    std::string name;
    uint32_t width = 0, height = 0;
    std::vector<bvhgb_pixel> pixels;
    std::vector<bvhgb_hit> hits;
    double ns = 0.0;
  };
  std::vector<Work> work;
  ~State();
};

class Command {
 public:
  virtual ~Command() = default;
  ErrorCode run(State &s);  // Command::run (lib/base/Command.cpp:35-69)
  virtual std::string name() const = 0;
  virtual std::string desc() const = 0;
  virtual uint64_t type() const = 0;
  virtual uint64_t required() const = 0;
  virtual void fromJSON(const Json &) {}
  virtual Json toJSON() const { return Json::object(); }

 protected:
  virtual ErrorCode setup(State &) { return ErrorCode::OK; }
  virtual ErrorCode runImpl(State &s) = 0;
  virtual void teardown(State &) {}
};

using CommandPtr = std::shared_ptr<Command>;
CommandPtr command_from_string(const std::string &name);  // fromString (src/main.cpp:66-95)
const std::vector<std::string> &command_names();

// Config (lib/base/Config.*): baseConfig {name, verbose, basePath, input[]} + commands[{cmd, options}].
struct Config {
  std::string name = "BVHTest default run";
  bool verbose = true;
  std::string basePath = ".";
  std::vector<std::string> input;
  std::vector<CommandPtr> commands;
  void fromJSON(const Json &j);
  Json toJSON() const;
};

// `bvhTest run CFG` (src/main.cpp:153-210): parse, rewrite the file with defaults filled in, run every
// command for every input; a command returning something other than OK/WARNING stops that input.
int run_config_file(const std::string &path, std::string *log = nullptr);

}  // namespace bvhgb::host
