// A small JSON reader and writer for the sl3d front end's configs: objects
// (keys kept sorted, so that a value's canonical text -- the run hash's input
// -- does not depend on the file's key order), arrays, strings, numbers,
// booleans and null. Errors throw std::invalid_argument with the offset.
#pragma once

#include <cmath>
#include <cstdio>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <variant>
#include <vector>

namespace sl3d::json {

struct Value;
using Object = std::map<std::string, Value>;
using Array = std::vector<Value>;

struct Value {
  std::variant<std::nullptr_t, bool, double, std::string, std::shared_ptr<Array>, std::shared_ptr<Object>> v;

  bool IsNull() const { return std::holds_alternative<std::nullptr_t>(v); }
  bool IsBool() const { return std::holds_alternative<bool>(v); }
  bool IsNumber() const { return std::holds_alternative<double>(v); }
  bool IsString() const { return std::holds_alternative<std::string>(v); }
  bool IsArray() const { return std::holds_alternative<std::shared_ptr<Array>>(v); }
  bool IsObject() const { return std::holds_alternative<std::shared_ptr<Object>>(v); }

  double Number(const std::string& what) const {
    if (!IsNumber()) throw std::invalid_argument(what + " must be a number");
    return std::get<double>(v);
  }
  bool Bool(const std::string& what) const {
    if (!IsBool()) throw std::invalid_argument(what + " must be true or false");
    return std::get<bool>(v);
  }
  const std::string& String(const std::string& what) const {
    if (!IsString()) throw std::invalid_argument(what + " must be a string");
    return std::get<std::string>(v);
  }
  const Array& Items(const std::string& what) const {
    if (!IsArray()) throw std::invalid_argument(what + " must be an array");
    return *std::get<std::shared_ptr<Array>>(v);
  }
  const Object& Members(const std::string& what) const {
    if (!IsObject()) throw std::invalid_argument(what + " must be an object");
    return *std::get<std::shared_ptr<Object>>(v);
  }
};

class Reader {
 public:
  explicit Reader(const std::string& text) : s_(text) {}

  Value Document() {
    Value out = Parse();
    Space();
    if (at_ != s_.size()) Fail("text after the value");
    return out;
  }

 private:
  const std::string& s_;
  size_t at_ = 0;

  [[noreturn]] void Fail(const std::string& what) const {
    throw std::invalid_argument("config: " + what + " at offset " + std::to_string(at_));
  }
  void Space() {
    while (at_ < s_.size() && (s_[at_] == ' ' || s_[at_] == '\n' || s_[at_] == '\r' || s_[at_] == '\t')) ++at_;
  }
  bool Take(char c) {
    Space();
    if (at_ < s_.size() && s_[at_] == c) {
      ++at_;
      return true;
    }
    return false;
  }
  void Expect(char c) {
    if (!Take(c)) Fail(std::string("'") + c + "' expected");
  }
  bool Word(const char* w) {
    const std::string word(w);
    if (s_.compare(at_, word.size(), word) == 0) {
      at_ += word.size();
      return true;
    }
    return false;
  }

  std::string Text() {
    Expect('"');
    std::string out;
    while (true) {
      if (at_ >= s_.size()) Fail("unterminated string");
      const char c = s_[at_++];
      if (c == '"') break;
      if (c != '\\') {
        out += c;
        continue;
      }
      if (at_ >= s_.size()) Fail("unterminated escape");
      const char e = s_[at_++];
      switch (e) {
        case '"': out += '"'; break;
        case '\\': out += '\\'; break;
        case '/': out += '/'; break;
        case 'n': out += '\n'; break;
        case 't': out += '\t'; break;
        case 'r': out += '\r'; break;
        case 'b': out += '\b'; break;
        case 'f': out += '\f'; break;
        default: Fail("an escape this reader does not take");
      }
    }
    return out;
  }

  Value Parse() {
    Space();
    if (at_ >= s_.size()) Fail("a value expected");
    const char c = s_[at_];
    Value out;
    if (c == '{') {
      ++at_;
      auto obj = std::make_shared<Object>();
      if (!Take('}')) {
        do {
          Space();
          const std::string key = Text();
          Expect(':');
          if (obj->count(key)) Fail("key \"" + key + "\" repeated");
          (*obj)[key] = Parse();
        } while (Take(','));
        Expect('}');
      }
      out.v = obj;
    } else if (c == '[') {
      ++at_;
      auto arr = std::make_shared<Array>();
      if (!Take(']')) {
        do arr->push_back(Parse());
        while (Take(','));
        Expect(']');
      }
      out.v = arr;
    } else if (c == '"') {
      out.v = Text();
    } else if (Word("true")) {
      out.v = true;
    } else if (Word("false")) {
      out.v = false;
    } else if (Word("null")) {
      out.v = nullptr;
    } else {
      const char* begin = s_.c_str() + at_;
      char* end = nullptr;
      const double d = std::strtod(begin, &end);
      if (end == begin) Fail("a value expected");
      at_ += static_cast<size_t>(end - begin);
      if (!std::isfinite(d)) Fail("a finite number expected");
      out.v = d;
    }
    return out;
  }
};

inline Value Parse(const std::string& text) { return Reader(text).Document(); }

// The canonical text of a value: keys sorted, numbers to 17 significant digits.
inline std::string Canonical(const Value& value) {
  if (value.IsNull()) return "null";
  if (value.IsBool()) return std::get<bool>(value.v) ? "true" : "false";
  if (value.IsNumber()) {
    char buf[40];
    std::snprintf(buf, sizeof(buf), "%.17g", std::get<double>(value.v));
    return buf;
  }
  if (value.IsString()) {
    std::string out = "\"";
    for (char c : std::get<std::string>(value.v)) {
      if (c == '"' || c == '\\') out += '\\';
      out += c;
    }
    return out + "\"";
  }
  if (value.IsArray()) {
    std::string out = "[";
    const auto& items = *std::get<std::shared_ptr<Array>>(value.v);
    for (size_t i = 0; i < items.size(); ++i) out += (i ? "," : "") + Canonical(items[i]);
    return out + "]";
  }
  std::string out = "{";
  bool first = true;
  for (const auto& [k, v] : *std::get<std::shared_ptr<Object>>(value.v)) {
    out += (first ? "\"" : ",\"") + k + "\":" + Canonical(v);
    first = false;
  }
  return out + "}";
}

}  // namespace sl3d::json
