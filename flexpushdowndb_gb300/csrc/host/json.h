// Minimal JSON value + recursive-descent parser for plan and expression specs.
// The reference deserialises plans and expressions with nlohmann::json
// (fpdb-expression-gandiva/src/Expression.cpp:52-148); this is the small
// subset the operator specs of this library need (objects, arrays, strings,
// numbers kept as both int64 and double, booleans, null).
#pragma once

#include <cstdint>
#include <cstdio>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace gfpdb::json {

struct Value {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  bool is_integer = false;
  int64_t i = 0;
  double d = 0.0;
  std::string s;
  std::vector<Value> a;
  std::vector<std::pair<std::string, Value>> o;  // insertion order kept

  bool contains(const std::string& key) const {
    if (kind != Object) return false;
    for (auto& kv : o)
      if (kv.first == key) return true;
    return false;
  }
  const Value& at(const std::string& key) const {
    if (kind != Object) throw std::runtime_error("JSON: '" + key + "' looked up in a non-object");
    for (auto& kv : o)
      if (kv.first == key) return kv.second;
    throw std::runtime_error("JSON: missing key '" + key + "'");
  }
  const std::string& str() const {
    if (kind != String) throw std::runtime_error("JSON: expected a string");
    return s;
  }
  int64_t integer() const {
    if (kind != Number || !is_integer) throw std::runtime_error("JSON: expected an integer");
    return i;
  }
  double number() const {
    if (kind != Number) throw std::runtime_error("JSON: expected a number");
    return is_integer ? static_cast<double>(i) : d;
  }
  bool boolean() const {
    if (kind != Bool) throw std::runtime_error("JSON: expected a boolean");
    return b;
  }
  const std::vector<Value>& array() const {
    if (kind != Array) throw std::runtime_error("JSON: expected an array");
    return a;
  }
  std::string get_str(const std::string& key, const std::string& dflt) const {
    return contains(key) ? at(key).str() : dflt;
  }
  int64_t get_int(const std::string& key, int64_t dflt) const {
    return contains(key) ? at(key).integer() : dflt;
  }
  double get_num(const std::string& key, double dflt) const {
    return contains(key) ? at(key).number() : dflt;
  }
  bool get_bool(const std::string& key, bool dflt) const {
    return contains(key) ? at(key).boolean() : dflt;
  }
  std::vector<std::string> str_list(const std::string& key) const {
    std::vector<std::string> out;
    if (!contains(key)) return out;
    for (auto& v : at(key).array()) out.push_back(v.str());
    return out;
  }
};

class Parser {
 public:
  explicit Parser(const std::string& text) : t_(text) {}

  Value parse() {
    Value v = value();
    ws();
    if (p_ != t_.size()) fail("trailing characters");
    return v;
  }

 private:
  const std::string& t_;
  size_t p_ = 0;
  int depth_ = 0;  // open objects and arrays: the descent is recursive, so bounded
  static constexpr int kMaxDepth = 512;

  [[noreturn]] void fail(const std::string& what) {
    throw std::runtime_error("JSON parse error at offset " + std::to_string(p_) + ": " + what);
  }
  void ws() {
    while (p_ < t_.size() && (t_[p_] == ' ' || t_[p_] == '\n' || t_[p_] == '\t' || t_[p_] == '\r')) ++p_;
  }
  char peek() {
    ws();
    if (p_ >= t_.size()) fail("unexpected end");
    return t_[p_];
  }
  void expect(char c) {
    if (peek() != c) fail(std::string("expected '") + c + "'");
    ++p_;
  }
  bool lit(const char* w) {
    size_t n = std::char_traits<char>::length(w);
    if (t_.compare(p_, n, w) == 0) {
      p_ += n;
      return true;
    }
    return false;
  }

  Value value() {
    char c = peek();
    Value v;
    if ((c == '{' || c == '[') && ++depth_ > kMaxDepth) fail("nesting deeper than 512 levels");
    struct Leave {
      int* d;
      bool on;
      ~Leave() {
        if (on) --*d;
      }
    } leave{&depth_, c == '{' || c == '['};
    if (c == '{') {
      v.kind = Value::Object;
      ++p_;
      if (peek() == '}') {
        ++p_;
        return v;
      }
      for (;;) {
        if (peek() != '"') fail("expected object key");
        std::string k = string_body();
        expect(':');
        v.o.emplace_back(std::move(k), value());
        char d = peek();
        ++p_;
        if (d == '}') break;
        if (d != ',') fail("expected ',' or '}'");
      }
    } else if (c == '[') {
      v.kind = Value::Array;
      ++p_;
      if (peek() == ']') {
        ++p_;
        return v;
      }
      for (;;) {
        v.a.push_back(value());
        char d = peek();
        ++p_;
        if (d == ']') break;
        if (d != ',') fail("expected ',' or ']'");
      }
    } else if (c == '"') {
      v.kind = Value::String;
      v.s = string_body();
    } else if (lit("true")) {
      v.kind = Value::Bool;
      v.b = true;
    } else if (lit("false")) {
      v.kind = Value::Bool;
      v.b = false;
    } else if (lit("null")) {
      v.kind = Value::Null;
    } else {
      v.kind = Value::Number;
      size_t start = p_;
      if (t_[p_] == '-' || t_[p_] == '+') ++p_;
      bool frac = false;
      while (p_ < t_.size()) {
        char d = t_[p_];
        if (d >= '0' && d <= '9') {
          ++p_;
        } else if (d == '.' || d == 'e' || d == 'E' || ((d == '-' || d == '+') && frac)) {
          frac = true;
          ++p_;
        } else {
          break;
        }
      }
      std::string num = t_.substr(start, p_ - start);
      if (num.empty() || num == "-" || num == "+") fail("bad number");
      if (!frac) {
        v.is_integer = true;
        v.i = std::stoll(num);
        v.d = static_cast<double>(v.i);
      } else {
        v.d = std::stod(num);
      }
    }
    return v;
  }

  std::string string_body() {
    expect('"');
    std::string out;
    while (p_ < t_.size() && t_[p_] != '"') {
      char c = t_[p_++];
      if (c == '\\') {
        if (p_ >= t_.size()) fail("bad escape");
        char e = t_[p_++];
        switch (e) {
          case 'n': out += '\n'; break;
          case 't': out += '\t'; break;
          case 'r': out += '\r'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'u': {
            if (p_ + 4 > t_.size()) fail("bad \\u escape");
            unsigned cp = std::stoul(t_.substr(p_, 4), nullptr, 16);
            p_ += 4;
            if (cp < 0x80) {
              out += static_cast<char>(cp);
            } else if (cp < 0x800) {
              out += static_cast<char>(0xC0 | (cp >> 6));
              out += static_cast<char>(0x80 | (cp & 0x3F));
            } else {
              out += static_cast<char>(0xE0 | (cp >> 12));
              out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
              out += static_cast<char>(0x80 | (cp & 0x3F));
            }
            break;
          }
          default: out += e;
        }
      } else {
        out += c;
      }
    }
    if (p_ >= t_.size()) fail("unterminated string");
    ++p_;
    return out;
  }
};

inline Value parse(const std::string& text) { return Parser(text).parse(); }

// The value as JSON text (object keys in insertion order; strings escaped,
// bytes >= 0x80 passed through as they are).
inline void dump_to(const Value& v, std::string& out) {
  switch (v.kind) {
    case Value::Null: out += "null"; break;
    case Value::Bool: out += v.b ? "true" : "false"; break;
    case Value::Number: {
      if (v.is_integer) {
        out += std::to_string(v.i);
      } else {
        char buf[32];
        std::snprintf(buf, sizeof(buf), "%.17g", v.d);
        out += buf;
      }
      break;
    }
    case Value::String: {
      out += '"';
      for (char c : v.s) {
        const unsigned char u = static_cast<unsigned char>(c);
        if (c == '"' || c == '\\') {
          out += '\\';
          out += c;
        } else if (u < 0x20) {
          char buf[8];
          std::snprintf(buf, sizeof(buf), "\\u%04x", u);
          out += buf;
        } else {
          out += c;
        }
      }
      out += '"';
      break;
    }
    case Value::Array: {
      out += '[';
      for (size_t k = 0; k < v.a.size(); ++k) {
        if (k) out += ',';
        dump_to(v.a[k], out);
      }
      out += ']';
      break;
    }
    case Value::Object: {
      out += '{';
      for (size_t k = 0; k < v.o.size(); ++k) {
        if (k) out += ',';
        Value key;
        key.kind = Value::String;
        key.s = v.o[k].first;
        dump_to(key, out);
        out += ':';
        dump_to(v.o[k].second, out);
      }
      out += '}';
      break;
    }
  }
}

inline std::string dump(const Value& v) {
  std::string out;
  dump_to(v, out);
  return out;
}

}  // namespace gfpdb::json
