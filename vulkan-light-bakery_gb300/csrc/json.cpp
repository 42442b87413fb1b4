// json.cpp -- parser and printer of json.h (host code).
#include "json.h"

#include <cerrno>
#include <cmath>
#include <cstdio>
#include <cstdlib>
#include <cstring>

namespace vlbj {
namespace {

struct Parser {
  const char* p;
  const char* end;
  std::string* err;
  int depth = 0;

  bool fail(const char* what) {
    if (err) *err = what;
    return false;
  }
  void ws() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
  }
  bool lit(const char* w) {
    const size_t n = std::strlen(w);
    if (size_t(end - p) < n || std::memcmp(p, w, n) != 0) return false;
    p += n;
    return true;
  }
  static void put_utf8(std::string& s, uint32_t c) {
    if (c < 0x80) {
      s += char(c);
    } else if (c < 0x800) {
      s += char(0xC0 | (c >> 6));
      s += char(0x80 | (c & 0x3F));
    } else if (c < 0x10000) {
      s += char(0xE0 | (c >> 12));
      s += char(0x80 | ((c >> 6) & 0x3F));
      s += char(0x80 | (c & 0x3F));
    } else {
      s += char(0xF0 | (c >> 18));
      s += char(0x80 | ((c >> 12) & 0x3F));
      s += char(0x80 | ((c >> 6) & 0x3F));
      s += char(0x80 | (c & 0x3F));
    }
  }
  bool hex4(uint32_t* v) {
    if (end - p < 4) return false;
    uint32_t x = 0;
    for (int i = 0; i < 4; ++i) {
      const char c = p[i];
      x <<= 4;
      if (c >= '0' && c <= '9') x |= uint32_t(c - '0');
      else if (c >= 'a' && c <= 'f') x |= uint32_t(c - 'a' + 10);
      else if (c >= 'A' && c <= 'F') x |= uint32_t(c - 'A' + 10);
      else return false;
    }
    p += 4;
    *v = x;
    return true;
  }
  // One UTF-8 sequence (validated: shortest form, no surrogates, <= U+10FFFF).
  bool utf8(std::string& s) {
    const unsigned char c0 = static_cast<unsigned char>(*p);
    int n;
    uint32_t cp;
    if (c0 < 0x80) { s += char(c0); ++p; return true; }
    if ((c0 & 0xE0) == 0xC0) { n = 2; cp = c0 & 0x1F; }
    else if ((c0 & 0xF0) == 0xE0) { n = 3; cp = c0 & 0x0F; }
    else if ((c0 & 0xF8) == 0xF0) { n = 4; cp = c0 & 0x07; }
    else return false;
    if (end - p < n) return false;
    for (int i = 1; i < n; ++i) {
      const unsigned char c = static_cast<unsigned char>(p[i]);
      if ((c & 0xC0) != 0x80) return false;
      cp = (cp << 6) | (c & 0x3F);
    }
    if ((n == 2 && cp < 0x80) || (n == 3 && cp < 0x800) || (n == 4 && cp < 0x10000) || cp > 0x10FFFF ||
        (cp >= 0xD800 && cp <= 0xDFFF))
      return false;
    s.append(p, size_t(n));
    p += n;
    return true;
  }
  bool string(std::string& s) {
    ++p;  // opening quote
    for (;;) {
      if (p >= end) return fail("unterminated string");
      const char c = *p;
      if (c == '"') { ++p; return true; }
      if (static_cast<unsigned char>(c) < 0x20) return fail("control character in string");
      if (c != '\\') {
        if (!utf8(s)) return fail("invalid UTF-8 in string");
        continue;
      }
      ++p;
      if (p >= end) return fail("bad escape");
      const char e = *p++;
      switch (e) {
        case '"': s += '"'; break;
        case '\\': s += '\\'; break;
        case '/': s += '/'; break;
        case 'b': s += '\b'; break;
        case 'f': s += '\f'; break;
        case 'n': s += '\n'; break;
        case 'r': s += '\r'; break;
        case 't': s += '\t'; break;
        case 'u': {
          uint32_t cp;
          if (!hex4(&cp)) return fail("bad \\u escape");
          if (cp >= 0xD800 && cp <= 0xDBFF) {
            uint32_t lo;
            if (end - p < 6 || p[0] != '\\' || p[1] != 'u') return fail("lone surrogate");
            p += 2;
            if (!hex4(&lo) || lo < 0xDC00 || lo > 0xDFFF) return fail("bad surrogate pair");
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          } else if (cp >= 0xDC00 && cp <= 0xDFFF) {
            return fail("lone surrogate");
          }
          put_utf8(s, cp);
          break;
        }
        default:
          return fail("bad escape");
      }
    }
  }
  bool number(Value* v) {
    const char* s0 = p;
    bool neg = false, is_float = false;
    if (*p == '-') { neg = true; ++p; }
    if (p >= end) return fail("bad number");
    if (*p == '0') {
      ++p;
    } else if (*p >= '1' && *p <= '9') {
      while (p < end && *p >= '0' && *p <= '9') ++p;
    } else {
      return fail("bad number");
    }
    if (p < end && *p == '.') {
      is_float = true;
      ++p;
      if (p >= end || !(*p >= '0' && *p <= '9')) return fail("bad number");
      while (p < end && *p >= '0' && *p <= '9') ++p;
    }
    if (p < end && (*p == 'e' || *p == 'E')) {
      is_float = true;
      ++p;
      if (p < end && (*p == '+' || *p == '-')) ++p;
      if (p >= end || !(*p >= '0' && *p <= '9')) return fail("bad number");
      while (p < end && *p >= '0' && *p <= '9') ++p;
    }
    const std::string tok(s0, size_t(p - s0));
    if (!is_float) {
      errno = 0;
      char* e = nullptr;
      if (neg) {
        const long long x = std::strtoll(tok.c_str(), &e, 10);
        if (errno == 0) { *v = Value::integer(x); return true; }
      } else {
        const unsigned long long x = std::strtoull(tok.c_str(), &e, 10);
        if (errno == 0) { *v = Value::uinteger(x); return true; }
      }
    }
    *v = Value::number(std::strtod(tok.c_str(), nullptr));  // out-of-range integers become doubles
    return true;
  }
  bool value(Value* v) {
    ws();
    if (p >= end) return fail("unexpected end");
    if (++depth > 512) return fail("nesting too deep");
    bool ok = true;
    const char c = *p;
    if (c == '{') {
      ++p;
      *v = Value::object();
      ws();
      if (p < end && *p == '}') {
        ++p;
      } else {
        for (;;) {
          ws();
          if (p >= end || *p != '"') { ok = fail("expected a key"); break; }
          std::string k;
          if (!string(k)) { ok = false; break; }
          ws();
          if (p >= end || *p != ':') { ok = fail("expected ':'"); break; }
          ++p;
          Value x;
          if (!value(&x)) { ok = false; break; }
          v->o[k] = std::move(x);  // a repeated key keeps its last value
          ws();
          if (p < end && *p == ',') { ++p; continue; }
          if (p < end && *p == '}') { ++p; break; }
          ok = fail("expected ',' or '}'");
          break;
        }
      }
    } else if (c == '[') {
      ++p;
      *v = Value::array();
      ws();
      if (p < end && *p == ']') {
        ++p;
      } else {
        for (;;) {
          Value x;
          if (!value(&x)) { ok = false; break; }
          v->a.push_back(std::move(x));
          ws();
          if (p < end && *p == ',') { ++p; continue; }
          if (p < end && *p == ']') { ++p; break; }
          ok = fail("expected ',' or ']'");
          break;
        }
      }
    } else if (c == '"') {
      *v = Value::string("");
      ok = string(v->s);
    } else if (c == '-' || (c >= '0' && c <= '9')) {
      ok = number(v);
    } else if (lit("true")) {
      *v = Value::boolean(true);
    } else if (lit("false")) {
      *v = Value::boolean(false);
    } else if (lit("null")) {
      *v = Value::null();
    } else {
      ok = fail("unexpected character");
    }
    --depth;
    return ok;
  }
};

void quote(const std::string& s, std::string& o) {
  o += '"';
  for (const char ch : s) {
    const unsigned char c = static_cast<unsigned char>(ch);
    switch (c) {
      case '"': o += "\\\""; break;
      case '\\': o += "\\\\"; break;
      case '\b': o += "\\b"; break;
      case '\f': o += "\\f"; break;
      case '\n': o += "\\n"; break;
      case '\r': o += "\\r"; break;
      case '\t': o += "\\t"; break;
      default:
        if (c < 0x20) {
          char b[8];
          std::snprintf(b, sizeof b, "\\u%04x", unsigned(c));
          o += b;
        } else {
          o += ch;
        }
    }
  }
  o += '"';
}

void dump_rec(const Value& v, std::string& o, int level) {
  switch (v.type) {
    case Value::kNull: o += "null"; return;
    case Value::kBool: o += v.b ? "true" : "false"; return;
    case Value::kInt: o += std::to_string(v.i); return;
    case Value::kUint: o += std::to_string(v.u); return;
    case Value::kFloat: o += format_double(v.f); return;
    case Value::kString: quote(v.s, o); return;
    case Value::kArray: {
      if (v.a.empty()) { o += "[]"; return; }
      o += "[\n";
      for (size_t i = 0; i < v.a.size(); ++i) {
        o.append(size_t(4 * (level + 1)), ' ');
        dump_rec(v.a[i], o, level + 1);
        o += i + 1 < v.a.size() ? ",\n" : "\n";
      }
      o.append(size_t(4 * level), ' ');
      o += ']';
      return;
    }
    case Value::kObject: {
      if (v.o.empty()) { o += "{}"; return; }
      o += "{\n";
      size_t i = 0;
      for (const auto& kv : v.o) {
        o.append(size_t(4 * (level + 1)), ' ');
        quote(kv.first, o);
        o += ": ";
        dump_rec(kv.second, o, level + 1);
        o += ++i < v.o.size() ? ",\n" : "\n";
      }
      o.append(size_t(4 * level), ' ');
      o += '}';
      return;
    }
  }
}

}  // namespace

bool parse(const char* text, size_t len, Value* out, std::string* err) {
  Parser ps{text, text + len, err};
  Value v;
  if (!ps.value(&v)) return false;
  ps.ws();
  if (ps.p != ps.end) return ps.fail("trailing characters");
  *out = std::move(v);
  return true;
}

std::string dump(const Value& v) {
  std::string o;
  dump_rec(v, o, 0);
  return o;
}

std::string format_double(double x) {
  if (!std::isfinite(x)) return "null";
  if (x == 0.0) return std::signbit(x) ? "-0.0" : "0.0";
  // shortest significand that reads back to x (correctly rounded at each length)
  char buf[40];
  for (int prec = 0; prec <= 16; ++prec) {
    std::snprintf(buf, sizeof buf, "%.*e", prec, x);
    if (std::strtod(buf, nullptr) == x) break;
  }
  // buf: [-]d[.ddd]e(+|-)XX
  std::string digits;
  const char* q = buf;
  std::string out;
  if (*q == '-') { out += '-'; ++q; }
  while (*q && *q != 'e') {
    if (*q != '.') digits += *q;
    ++q;
  }
  const int e10 = std::atoi(q + 1);
  while (digits.size() > 1 && digits.back() == '0') digits.pop_back();
  const int k = int(digits.size());
  const int n = e10 + 1;  // position of the decimal point from the first digit
  constexpr int kMinExp = -4, kMaxExp = 15;
  if (k <= n && n <= kMaxExp) {
    out += digits;
    out.append(size_t(n - k), '0');
    out += ".0";
  } else if (0 < n && n <= kMaxExp) {
    out += digits.substr(0, size_t(n));
    out += '.';
    out += digits.substr(size_t(n));
  } else if (kMinExp < n && n <= 0) {
    out += "0.";
    out.append(size_t(-n), '0');
    out += digits;
  } else {
    out += digits[0];
    if (k > 1) {
      out += '.';
      out += digits.substr(1);
    }
    int e = n - 1;
    out += 'e';
    out += e < 0 ? '-' : '+';
    if (e < 0) e = -e;
    char eb[8];
    std::snprintf(eb, sizeof eb, "%02d", e);
    out += eb;
  }
  return out;
}

}  // namespace vlbj
