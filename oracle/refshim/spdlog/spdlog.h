// Test infrastructure only: the named-logger calls the reference's CPU files make
// (get / stdout_color_mt and info / warn / error / debug with "{}" formatting). Written here
// because the reference's logging submodule is empty. Messages go to stderr when the environment
// variable BVHREF_LOG is set and are dropped otherwise, so the reference code runs quietly when it
// serves as the oracle's pin.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <mutex>
#include <string>

#include "../fmt/format.h"

namespace spdlog {

class logger {
 public:
  explicit logger(std::string name) : name_(std::move(name)) {}
  template <typename... A>
  void info(const std::string &f, A &&...a) { emit("info", fmt::format(f, std::forward<A>(a)...)); }
  template <typename... A>
  void warn(const std::string &f, A &&...a) { emit("warn", fmt::format(f, std::forward<A>(a)...)); }
  template <typename... A>
  void error(const std::string &f, A &&...a) { emit("error", fmt::format(f, std::forward<A>(a)...)); }
  template <typename... A>
  void debug(const std::string &f, A &&...a) { emit("debug", fmt::format(f, std::forward<A>(a)...)); }
  template <typename... A>
  void critical(const std::string &f, A &&...a) { emit("critical", fmt::format(f, std::forward<A>(a)...)); }

 private:
  void emit(const char *level, const std::string &msg) {
    if (std::getenv("BVHREF_LOG")) std::fprintf(stderr, "[%s] [%s] %s\n", name_.c_str(), level, msg.c_str());
  }
  std::string name_;
};

namespace shim_detail {
inline std::map<std::string, std::shared_ptr<logger>> &registry() {
  static std::map<std::string, std::shared_ptr<logger>> r;
  return r;
}
inline std::mutex &registry_mutex() {
  static std::mutex m;
  return m;
}
}  // namespace shim_detail

inline std::shared_ptr<logger> get(const std::string &name) {
  std::lock_guard<std::mutex> g(shim_detail::registry_mutex());
  auto it = shim_detail::registry().find(name);
  return it == shim_detail::registry().end() ? nullptr : it->second;
}

inline std::shared_ptr<logger> stdout_color_mt(const std::string &name) {
  std::lock_guard<std::mutex> g(shim_detail::registry_mutex());
  auto &slot = shim_detail::registry()[name];
  if (!slot) slot = std::make_shared<logger>(name);
  return slot;
}

}  // namespace spdlog
