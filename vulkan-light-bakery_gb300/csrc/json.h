// json.h -- a small JSON document model for the glTF entry points.
//
// The reference reads and writes glTF with nlohmann::json (third-party,
// nlohmann/json, header-only; src/baker/light_baker.cpp:375-401,
// src/scene_manager.cpp:613-648).  Its observable behaviour is restated
// here, not its code:
//   * objects keep their keys sorted by byte value (nlohmann's default
//     object type is std::map); a repeated key keeps its last value;
//   * numbers without '.', 'e' or 'E' parse as unsigned (non-negative) or
//     signed 64-bit integers, everything else as double;
//   * `out << std::setw(4) << j` prints with 4-space indentation, ": " after
//     keys, one element per line, "[]" / "{}" when empty;
//   * strings escape '"', '\\', the short forms \b \f \n \r \t and other
//     control characters as \u00xx (lowercase hex); other bytes (UTF-8) are
//     written as they are;
//   * doubles print as the shortest decimal that reads back to the same
//     value: fixed notation with ".0" for integral values when the decimal
//     point falls within 17 digits, "0.000ddd" down to 1e-4, else
//     d.ddde+XX with at least two exponent digits; NaN and infinities as
//     null.
#pragma once

#include <cstdint>
#include <map>
#include <memory>
#include <string>
#include <vector>

namespace vlbj {

struct Value {
  enum Type { kNull, kBool, kInt, kUint, kFloat, kString, kArray, kObject } type = kNull;
  bool b = false;
  int64_t i = 0;
  uint64_t u = 0;
  double f = 0.0;
  std::string s;
  std::vector<Value> a;
  std::map<std::string, Value> o;

  static Value null() { return Value(); }
  static Value boolean(bool v) { Value x; x.type = kBool; x.b = v; return x; }
  static Value integer(int64_t v) { Value x; x.type = kInt; x.i = v; return x; }
  static Value uinteger(uint64_t v) { Value x; x.type = kUint; x.u = v; return x; }
  static Value number(double v) { Value x; x.type = kFloat; x.f = v; return x; }
  static Value string(std::string v) { Value x; x.type = kString; x.s = std::move(v); return x; }
  static Value array() { Value x; x.type = kArray; return x; }
  static Value object() { Value x; x.type = kObject; return x; }

  bool is_number() const { return type == kInt || type == kUint || type == kFloat; }
  double as_double() const { return type == kFloat ? f : type == kInt ? double(i) : type == kUint ? double(u) : 0.0; }
  int64_t as_int() const { return type == kInt ? i : type == kUint ? int64_t(u) : type == kFloat ? int64_t(f) : 0; }
  const Value* get(const std::string& k) const {
    if (type != kObject) return nullptr;
    auto it = o.find(k);
    return it == o.end() ? nullptr : &it->second;
  }
  const Value* at(size_t idx) const { return type == kArray && idx < a.size() ? &a[idx] : nullptr; }
};

// Parses a whole document (RFC 8259; surrounding whitespace allowed).
// Returns false with a message on malformed input.
bool parse(const char* text, size_t len, Value* out, std::string* err);
// Pretty print, 4-space indentation (no trailing newline).
std::string dump(const Value& v);
// The double formatting rule above.
std::string format_double(double x);

}  // namespace vlbj
