// Minimal JSON value: parser (recursive descent) and writer. Mutating accessors copy shared
// storage first, so copies of a Json never alias.
#include "json.hpp"

#include <cmath>
#include <cstdio>
#include <cstdlib>

namespace bvhgb::host {

namespace {

struct Parser {
  const std::string &s;
  size_t i = 0;

  [[noreturn]] void fail(const char *what) const {
    throw JsonError(std::string("JSON parse error at offset ") + std::to_string(i) + ": " + what);
  }
  void ws() {
    while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r')) ++i;
  }
  bool lit(const char *w) {
    size_t n = 0;
    while (w[n]) ++n;
    if (s.compare(i, n, w) == 0) {
      i += n;
      return true;
    }
    return false;
  }
  static void put_utf8(std::string &out, uint32_t cp) {
    if (cp < 0x80) {
      out += (char)cp;
    } else if (cp < 0x800) {
      out += (char)(0xC0 | (cp >> 6));
      out += (char)(0x80 | (cp & 0x3F));
    } else if (cp < 0x10000) {
      out += (char)(0xE0 | (cp >> 12));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    } else {
      out += (char)(0xF0 | (cp >> 18));
      out += (char)(0x80 | ((cp >> 12) & 0x3F));
      out += (char)(0x80 | ((cp >> 6) & 0x3F));
      out += (char)(0x80 | (cp & 0x3F));
    }
  }
  uint32_t hex4() {
    if (i + 4 > s.size()) fail("short \\u escape");
    uint32_t v = 0;
    for (int k = 0; k < 4; ++k) {
      char c = s[i++];
      v <<= 4;
      if (c >= '0' && c <= '9') v |= (uint32_t)(c - '0');
      else if (c >= 'a' && c <= 'f') v |= (uint32_t)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') v |= (uint32_t)(c - 'A' + 10);
      else fail("bad \\u escape");
    }
    return v;
  }
  std::string str() {
    if (i >= s.size() || s[i] != '"') fail("expected string");
    ++i;
    std::string out;
    while (true) {
      if (i >= s.size()) fail("unterminated string");
      char c = s[i++];
      if (c == '"') break;
      if ((unsigned char)c < 0x20) fail("control character in string");
      if (c != '\\') {
        out += c;
        continue;
      }
      if (i >= s.size()) fail("bad escape");
      char e = s[i++];
      switch (e) {
        case '"': out += '"'; break;
        case '\\': out += '\\'; break;
        case '/': out += '/'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        case 'n': out += '\n'; break;
        case 'r': out += '\r'; break;
        case 't': out += '\t'; break;
        case 'u': {
          uint32_t cp = hex4();
          if (cp >= 0xD800 && cp < 0xDC00 && i + 6 <= s.size() && s[i] == '\\' && s[i + 1] == 'u') {
            i += 2;
            uint32_t lo = hex4();
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          }
          put_utf8(out, cp);
          break;
        }
        default: fail("bad escape");
      }
    }
    return out;
  }
  Json number() {
    size_t start = i;
    if (s[i] == '-') ++i;
    if (i >= s.size() || !(s[i] >= '0' && s[i] <= '9')) fail("bad number");
    while (i < s.size() && ((s[i] >= '0' && s[i] <= '9') || s[i] == '.' || s[i] == 'e' || s[i] == 'E' ||
                            s[i] == '+' || s[i] == '-'))
      ++i;
    std::string tok = s.substr(start, i - start);
    char *end = nullptr;
    double v = std::strtod(tok.c_str(), &end);
    if (!end || *end) fail("bad number");
    return Json(v);
  }
  Json value(int depth) {
    if (depth > 512) fail("nesting too deep");
    ws();
    if (i >= s.size()) fail("unexpected end");
    char c = s[i];
    if (c == '{') {
      ++i;
      JsonObject o;
      ws();
      if (i < s.size() && s[i] == '}') {
        ++i;
        return Json(std::move(o));
      }
      while (true) {
        ws();
        std::string k = str();
        ws();
        if (i >= s.size() || s[i] != ':') fail("expected ':'");
        ++i;
        o[k] = value(depth + 1);
        ws();
        if (i < s.size() && s[i] == ',') {
          ++i;
          continue;
        }
        if (i < s.size() && s[i] == '}') {
          ++i;
          break;
        }
        fail("expected ',' or '}'");
      }
      return Json(std::move(o));
    }
    if (c == '[') {
      ++i;
      JsonArray a;
      ws();
      if (i < s.size() && s[i] == ']') {
        ++i;
        return Json(std::move(a));
      }
      while (true) {
        a.push_back(value(depth + 1));
        ws();
        if (i < s.size() && s[i] == ',') {
          ++i;
          continue;
        }
        if (i < s.size() && s[i] == ']') {
          ++i;
          break;
        }
        fail("expected ',' or ']'");
      }
      return Json(std::move(a));
    }
    if (c == '"') return Json(str());
    if (lit("true")) return Json(true);
    if (lit("false")) return Json(false);
    if (lit("null")) return Json();
    return number();
  }
};

void escape(std::string &out, const std::string &v) {
  out += '"';
  for (unsigned char c : v) {
    switch (c) {
      case '"': out += "\\\""; break;
      case '\\': out += "\\\\"; break;
      case '\n': out += "\\n"; break;
      case '\r': out += "\\r"; break;
      case '\t': out += "\\t"; break;
      default:
        if (c < 0x20) {
          char buf[8];
          std::snprintf(buf, sizeof(buf), "\\u%04x", c);
          out += buf;
        } else {
          out += (char)c;
        }
    }
  }
  out += '"';
}

}  // namespace

Json Json::parse(const std::string &text) {
  Parser p{text};
  Json v = p.value(0);
  p.ws();
  if (p.i != text.size()) p.fail("trailing characters");
  return v;
}

bool Json::as_bool() const {
  if (type_ != Type::Bool) throw JsonError("not a boolean");
  return b_;
}
double Json::as_number() const {
  if (type_ != Type::Number) throw JsonError("not a number");
  return d_;
}
const std::string &Json::as_string() const {
  if (type_ != Type::String) throw JsonError("not a string");
  return *s_;
}
const JsonArray &Json::as_array() const {
  if (type_ != Type::Array) throw JsonError("not an array");
  return *a_;
}
JsonArray &Json::as_array() {
  if (type_ != Type::Array) throw JsonError("not an array");
  if (a_.use_count() > 1) a_ = std::make_shared<JsonArray>(*a_);
  return *a_;
}
const JsonObject &Json::as_object() const {
  if (type_ != Type::Object) throw JsonError("not an object");
  return *o_;
}
JsonObject &Json::as_object() {
  if (type_ != Type::Object) throw JsonError("not an object");
  if (o_.use_count() > 1) o_ = std::make_shared<JsonObject>(*o_);
  return *o_;
}

bool Json::contains(const std::string &key) const { return type_ == Type::Object && o_->count(key) != 0; }

const Json &Json::at(const std::string &key) const {
  if (type_ != Type::Object) throw JsonError("not an object (looking up '" + key + "')");
  auto it = o_->find(key);
  if (it == o_->end()) throw JsonError("missing key '" + key + "'");
  return it->second;
}

Json &Json::operator[](const std::string &key) {
  if (type_ == Type::Null) *this = object();
  return as_object()[key];
}

void Json::push_back(Json v) {
  if (type_ == Type::Null) *this = array();
  as_array().push_back(std::move(v));
}

size_t Json::size() const {
  if (type_ == Type::Array) return a_->size();
  if (type_ == Type::Object) return o_->size();
  return 0;
}

bool Json::value(const std::string &key, bool def) const {
  if (!contains(key)) return def;
  const Json &v = at(key);
  return v.is_bool() ? v.b_ : (v.is_number() ? v.d_ != 0.0 : def);
}
double Json::value(const std::string &key, double def) const {
  if (!contains(key)) return def;
  const Json &v = at(key);
  return v.is_number() ? v.d_ : def;
}
float Json::value(const std::string &key, float def) const { return (float)value(key, (double)def); }
uint32_t Json::value(const std::string &key, uint32_t def) const {
  double d = value(key, (double)def);
  return d < 0 ? 0u : (uint32_t)d;
}
int Json::value(const std::string &key, int def) const { return (int)value(key, (double)def); }
std::string Json::value(const std::string &key, const std::string &def) const {
  if (!contains(key)) return def;
  const Json &v = at(key);
  return v.is_string() ? *v.s_ : def;
}
Json Json::value(const std::string &key, const Json &def) const { return contains(key) ? at(key) : def; }

void Json::dump_to(std::string &out, int indent, int level) const {
  auto nl = [&](int l) {
    if (indent < 0) return;
    out += '\n';
    out.append((size_t)(indent * l), ' ');
  };
  switch (type_) {
    case Type::Null: out += "null"; break;
    case Type::Bool: out += b_ ? "true" : "false"; break;
    case Type::Number: {
      if (std::isfinite(d_) && d_ == std::floor(d_) && std::fabs(d_) < 9.007199254740992e15) {
        out += std::to_string((long long)d_);
      } else if (!std::isfinite(d_)) {
        out += "null";
      } else {
        char buf[32];
        std::snprintf(buf, sizeof(buf), "%.17g", d_);
        out += buf;
      }
      break;
    }
    case Type::String: escape(out, *s_); break;
    case Type::Array: {
      out += '[';
      if (a_->empty()) {
        out += ']';
        break;
      }
      bool first = true;
      for (const auto &v : *a_) {
        if (!first) out += ',';
        first = false;
        nl(level + 1);
        v.dump_to(out, indent, level + 1);
      }
      nl(level);
      out += ']';
      break;
    }
    case Type::Object: {
      out += '{';
      if (o_->empty()) {
        out += '}';
        break;
      }
      bool first = true;
      for (const auto &kv : *o_) {
        if (!first) out += ',';
        first = false;
        nl(level + 1);
        escape(out, kv.first);
        out += indent < 0 ? ":" : ": ";
        kv.second.dump_to(out, indent, level + 1);
      }
      nl(level);
      out += '}';
      break;
    }
  }
}

std::string Json::dump(int indent) const {
  std::string out;
  dump_to(out, indent, 0);
  return out;
}

}  // namespace bvhgb::host
