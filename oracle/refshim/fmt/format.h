// Test infrastructure only: the small part of a "{}"-placeholder string formatter that the
// reference's CPU files call (fmt::format with positional "{}" fields and width / alignment /
// precision specs such as "{:<8}" or "{:<6.5}"). Written here because the reference's formatter
// submodule is empty; it only has to make the reference's sources compile and produce readable
// log lines in oracle/_ref.
#pragma once

#include <iomanip>
#include <sstream>
#include <string>
#include <utility>

namespace fmt {
namespace shim_detail {

inline void apply_spec(std::ostringstream &os, const std::string &spec) {
  std::size_t i = 0;
  if (i < spec.size() && (spec[i] == '<' || spec[i] == '>' || spec[i] == '^')) {
    os << (spec[i] == '<' ? std::left : std::right);
    ++i;
  }
  int width = 0;
  while (i < spec.size() && spec[i] >= '0' && spec[i] <= '9') width = width * 10 + (spec[i++] - '0');
  if (width) os << std::setw(width);
  if (i < spec.size() && spec[i] == '.') {
    ++i;
    int prec = 0;
    while (i < spec.size() && spec[i] >= '0' && spec[i] <= '9') prec = prec * 10 + (spec[i++] - '0');
    os << std::setprecision(prec);
  }
}

inline void format_rest(std::string &out, const std::string &f, std::size_t pos) { out.append(f, pos, std::string::npos); }

template <typename A, typename... R>
void format_rest(std::string &out, const std::string &f, std::size_t pos, A &&a, R &&...rest) {
  std::size_t open = f.find('{', pos);
  if (open == std::string::npos) {
    out.append(f, pos, std::string::npos);
    return;
  }
  std::size_t close = f.find('}', open);
  if (close == std::string::npos) {
    out.append(f, pos, std::string::npos);
    return;
  }
  out.append(f, pos, open - pos);
  std::string spec = f.substr(open + 1, close - open - 1);
  if (!spec.empty() && spec[0] == ':') spec.erase(0, 1);
  std::ostringstream os;
  apply_spec(os, spec);
  os << a;
  out += os.str();
  format_rest(out, f, close + 1, std::forward<R>(rest)...);
}

}  // namespace shim_detail

template <typename... A>
std::string format(const std::string &f, A &&...args) {
  std::string out;
  shim_detail::format_rest(out, f, 0, std::forward<A>(args)...);
  return out;
}

}  // namespace fmt
