// json_min.hpp -- a small JSON reader for HDoG parameter files (objects, arrays,
// strings with escapes, numbers, true/false/null).  Repeated keys keep the last value,
// which is how the reference's '#' comment keys behave under nlohmann::json.
#pragma once
#include <cstdlib>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace hdog {
namespace json {

struct Value {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0.0;
  std::string str;
  std::vector<Value> arr;
  std::map<std::string, Value> obj;

  const Value *get(const std::string &k) const {
    if (kind != Object) return nullptr;
    auto it = obj.find(k);
    return it == obj.end() ? nullptr : &it->second;
  }
};

class Parser {
 public:
  explicit Parser(const std::string &s) : s_(s) {}
  bool parse(Value &out, std::string &err) {
    pos_ = 0;
    if (!value(out)) { err = err_.empty() ? "malformed JSON" : err_; return false; }
    ws();
    if (pos_ != s_.size()) { err = "trailing characters after JSON value"; return false; }
    return true;
  }

 private:
  const std::string &s_;
  size_t pos_ = 0;
  std::string err_;

  void ws() {
    while (pos_ < s_.size() && (s_[pos_] == ' ' || s_[pos_] == '\t' || s_[pos_] == '\n' || s_[pos_] == '\r')) pos_++;
  }
  bool fail(const char *m) {
    if (err_.empty()) err_ = std::string(m) + " at offset " + std::to_string(pos_);
    return false;
  }
  bool lit(const char *w) {
    size_t n = 0;
    while (w[n]) n++;
    if (s_.compare(pos_, n, w) != 0) return fail("unexpected token");
    pos_ += n;
    return true;
  }
  static void utf8(std::string &o, unsigned cp) {
    if (cp < 0x80) o += (char)cp;
    else if (cp < 0x800) { o += (char)(0xC0 | (cp >> 6)); o += (char)(0x80 | (cp & 0x3F)); }
    else if (cp < 0x10000) { o += (char)(0xE0 | (cp >> 12)); o += (char)(0x80 | ((cp >> 6) & 0x3F)); o += (char)(0x80 | (cp & 0x3F)); }
    else { o += (char)(0xF0 | (cp >> 18)); o += (char)(0x80 | ((cp >> 12) & 0x3F)); o += (char)(0x80 | ((cp >> 6) & 0x3F)); o += (char)(0x80 | (cp & 0x3F)); }
  }
  bool hex4(unsigned &cp) {
    if (pos_ + 4 > s_.size()) return fail("short \\u escape");
    cp = 0;
    for (int i = 0; i < 4; i++) {
      char c = s_[pos_++];
      cp <<= 4;
      if (c >= '0' && c <= '9') cp |= (unsigned)(c - '0');
      else if (c >= 'a' && c <= 'f') cp |= (unsigned)(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') cp |= (unsigned)(c - 'A' + 10);
      else return fail("bad \\u escape");
    }
    return true;
  }
  bool string(std::string &o) {
    if (s_[pos_] != '"') return fail("expected string");
    pos_++;
    while (pos_ < s_.size()) {
      char c = s_[pos_++];
      if (c == '"') return true;
      if (c != '\\') { o += c; continue; }
      if (pos_ >= s_.size()) break;
      char e = s_[pos_++];
      switch (e) {
        case '"': o += '"'; break;
        case '\\': o += '\\'; break;
        case '/': o += '/'; break;
        case 'b': o += '\b'; break;
        case 'f': o += '\f'; break;
        case 'n': o += '\n'; break;
        case 'r': o += '\r'; break;
        case 't': o += '\t'; break;
        case 'u': {
          unsigned cp;
          if (!hex4(cp)) return false;
          if (cp >= 0xD800 && cp < 0xDC00 && pos_ + 6 <= s_.size() && s_[pos_] == '\\' && s_[pos_ + 1] == 'u') {
            pos_ += 2;
            unsigned lo;
            if (!hex4(lo)) return false;
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          }
          utf8(o, cp);
          break;
        }
        default: return fail("bad escape");
      }
    }
    return fail("unterminated string");
  }
  bool number(Value &v) {
    const char *b = s_.c_str() + pos_;
    char *e = nullptr;
    v.num = std::strtod(b, &e);
    if (e == b) return fail("bad number");
    pos_ += (size_t)(e - b);
    v.kind = Value::Number;
    return true;
  }
  bool value(Value &v) {
    ws();
    if (pos_ >= s_.size()) return fail("unexpected end");
    const char c = s_[pos_];
    if (c == '{') {
      pos_++;
      v.kind = Value::Object;
      ws();
      if (pos_ < s_.size() && s_[pos_] == '}') { pos_++; return true; }
      while (true) {
        ws();
        std::string k;
        if (pos_ >= s_.size() || !string(k)) return fail("expected key");
        ws();
        if (pos_ >= s_.size() || s_[pos_] != ':') return fail("expected ':'");
        pos_++;
        Value item;
        if (!value(item)) return false;
        v.obj[k] = std::move(item);
        ws();
        if (pos_ < s_.size() && s_[pos_] == ',') { pos_++; continue; }
        if (pos_ < s_.size() && s_[pos_] == '}') { pos_++; return true; }
        return fail("expected ',' or '}'");
      }
    }
    if (c == '[') {
      pos_++;
      v.kind = Value::Array;
      ws();
      if (pos_ < s_.size() && s_[pos_] == ']') { pos_++; return true; }
      while (true) {
        Value item;
        if (!value(item)) return false;
        v.arr.push_back(std::move(item));
        ws();
        if (pos_ < s_.size() && s_[pos_] == ',') { pos_++; continue; }
        if (pos_ < s_.size() && s_[pos_] == ']') { pos_++; return true; }
        return fail("expected ',' or ']'");
      }
    }
    if (c == '"') { v.kind = Value::String; return string(v.str); }
    if (c == 't') { v.kind = Value::Bool; v.b = true; return lit("true"); }
    if (c == 'f') { v.kind = Value::Bool; v.b = false; return lit("false"); }
    if (c == 'n') { v.kind = Value::Null; return lit("null"); }
    return number(v);
  }
};

}  // namespace json
}  // namespace hdog
