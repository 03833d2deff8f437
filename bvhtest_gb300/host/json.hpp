// Minimal JSON value for the command configs and the IO formats: null, bool, number, string,
// array, object (keys kept sorted, as BVHTest's configs are written). Parsing is strict RFC 8259
// apart from accepting a trailing newline; numbers are held as double (exact for 53-bit ints).
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace bvhgb::host {

class Json;
using JsonArray = std::vector<Json>;
using JsonObject = std::map<std::string, Json>;

struct JsonError : std::runtime_error {
  using std::runtime_error::runtime_error;
};

class Json {
 public:
  enum class Type { Null, Bool, Number, String, Array, Object };

  Json() = default;
  Json(std::nullptr_t) {}
  Json(bool b) : type_(Type::Bool), b_(b) {}
  Json(double d) : type_(Type::Number), d_(d) {}
  Json(float d) : type_(Type::Number), d_(d) {}
  Json(int v) : type_(Type::Number), d_(v) {}
  Json(int64_t v) : type_(Type::Number), d_((double)v) {}
  Json(uint32_t v) : type_(Type::Number), d_(v) {}
  Json(uint64_t v) : type_(Type::Number), d_((double)v) {}
  Json(const char *s) : type_(Type::String), s_(std::make_shared<std::string>(s)) {}
  Json(std::string s) : type_(Type::String), s_(std::make_shared<std::string>(std::move(s))) {}
  Json(JsonArray a) : type_(Type::Array), a_(std::make_shared<JsonArray>(std::move(a))) {}
  Json(JsonObject o) : type_(Type::Object), o_(std::make_shared<JsonObject>(std::move(o))) {}

  static Json object() { return Json(JsonObject{}); }
  static Json array() { return Json(JsonArray{}); }
  static Json parse(const std::string &text);

  Type type() const { return type_; }
  bool is_null() const { return type_ == Type::Null; }
  bool is_bool() const { return type_ == Type::Bool; }
  bool is_number() const { return type_ == Type::Number; }
  bool is_string() const { return type_ == Type::String; }
  bool is_array() const { return type_ == Type::Array; }
  bool is_object() const { return type_ == Type::Object; }

  bool as_bool() const;
  double as_number() const;
  const std::string &as_string() const;
  const JsonArray &as_array() const;
  JsonArray &as_array();
  const JsonObject &as_object() const;
  JsonObject &as_object();

  bool contains(const std::string &key) const;
  const Json &at(const std::string &key) const;  // throws JsonError when missing
  Json &operator[](const std::string &key);      // creates an object / member
  void push_back(Json v);
  size_t size() const;

  // nlohmann-style value(key, default): the member converted to T, or the default when absent.
  bool value(const std::string &key, bool def) const;
  double value(const std::string &key, double def) const;
  float value(const std::string &key, float def) const;
  uint32_t value(const std::string &key, uint32_t def) const;
  int value(const std::string &key, int def) const;
  std::string value(const std::string &key, const std::string &def) const;
  std::string value(const std::string &key, const char *def) const { return value(key, std::string(def)); }
  Json value(const std::string &key, const Json &def) const;

  std::string dump(int indent = -1) const;

 private:
  void dump_to(std::string &out, int indent, int level) const;
  Type type_ = Type::Null;
  bool b_ = false;
  double d_ = 0.0;
  std::shared_ptr<std::string> s_;
  std::shared_ptr<JsonArray> a_;
  std::shared_ptr<JsonObject> o_;
};

}  // namespace bvhgb::host
