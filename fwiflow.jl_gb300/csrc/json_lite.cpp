// Minimal JSON reader; see json_lite.h.
#include "json_lite.h"

#include <cstdlib>
#include <cstring>
#include <fstream>

namespace fwigb {
namespace {

struct Parser {
  const char* p;
  const char* end;
  std::string err;

  void ws() {
    while (p < end && (*p == ' ' || *p == '\t' || *p == '\n' || *p == '\r')) ++p;
  }
  bool fail(const char* m) {
    if (err.empty()) err = m;
    return false;
  }
  bool lit(const char* s) {
    size_t n = std::strlen(s);
    if (static_cast<size_t>(end - p) < n || std::strncmp(p, s, n) != 0) return false;
    p += n;
    return true;
  }
  bool value(JValue& v, int depth) {
    if (depth > 64) return fail("JSON nested too deeply");
    ws();
    if (p >= end) return fail("unexpected end of JSON");
    char c = *p;
    if (c == '{') return object(v, depth);
    if (c == '[') return array(v, depth);
    if (c == '"') {
      v.kind = JValue::String;
      return string(v.str);
    }
    if (lit("true")) {
      v.kind = JValue::Bool;
      v.b = true;
      return true;
    }
    if (lit("false")) {
      v.kind = JValue::Bool;
      v.b = false;
      return true;
    }
    if (lit("null")) {
      v.kind = JValue::Null;
      return true;
    }
    return number(v);
  }
  bool number(JValue& v) {
    const char* s = p;
    if (p < end && (*p == '-' || *p == '+')) ++p;
    bool frac = false;
    while (p < end && ((*p >= '0' && *p <= '9') || *p == '.' || *p == 'e' || *p == 'E' || *p == '-' || *p == '+')) {
      if (*p == '.' || *p == 'e' || *p == 'E') frac = true;
      ++p;
    }
    if (p == s) return fail("invalid JSON value");
    std::string tok(s, p);
    char* q = nullptr;
    double d = std::strtod(tok.c_str(), &q);
    if (!q || *q != '\0') return fail("invalid JSON number");
    v.kind = JValue::Number;
    v.num = d;
    v.is_integer = !frac;
    return true;
  }
  bool string(std::string& out) {
    ++p;  // opening quote
    out.clear();
    while (p < end && *p != '"') {
      if (*p == '\\') {
        ++p;
        if (p >= end) return fail("bad escape");
        switch (*p) {
          case '"': out += '"'; break;
          case '\\': out += '\\'; break;
          case '/': out += '/'; break;
          case 'b': out += '\b'; break;
          case 'f': out += '\f'; break;
          case 'n': out += '\n'; break;
          case 'r': out += '\r'; break;
          case 't': out += '\t'; break;
          case 'u': {
            if (end - p < 5) return fail("bad \\u escape");
            unsigned cp = static_cast<unsigned>(std::strtoul(std::string(p + 1, p + 5).c_str(), nullptr, 16));
            p += 4;
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
          default: return fail("bad escape");
        }
        ++p;
      } else {
        out += *p++;
      }
    }
    if (p >= end) return fail("unterminated string");
    ++p;
    return true;
  }
  bool array(JValue& v, int depth) {
    ++p;
    v.kind = JValue::Array;
    ws();
    if (p < end && *p == ']') {
      ++p;
      return true;
    }
    while (true) {
      v.arr.emplace_back();
      if (!value(v.arr.back(), depth + 1)) return false;
      ws();
      if (p < end && *p == ',') {
        ++p;
        continue;
      }
      if (p < end && *p == ']') {
        ++p;
        return true;
      }
      return fail("expected , or ] in array");
    }
  }
  bool object(JValue& v, int depth) {
    ++p;
    v.kind = JValue::Object;
    ws();
    if (p < end && *p == '}') {
      ++p;
      return true;
    }
    while (true) {
      ws();
      if (p >= end || *p != '"') return fail("expected key string");
      std::string key;
      if (!string(key)) return false;
      ws();
      if (p >= end || *p != ':') return fail("expected :");
      ++p;
      JValue child;
      if (!value(child, depth + 1)) return false;
      v.obj[key] = std::move(child);
      ws();
      if (p < end && *p == ',') {
        ++p;
        continue;
      }
      if (p < end && *p == '}') {
        ++p;
        return true;
      }
      return fail("expected , or } in object");
    }
  }
};

}  // namespace

bool json_parse(const std::string& text, JValue& out, std::string& err) {
  Parser ps{text.data(), text.data() + text.size(), {}};
  if (!ps.value(out, 0)) {
    err = ps.err;
    return false;
  }
  return true;
}

bool json_read_first_line(const std::string& path, JValue& out, std::string& err) {
  std::ifstream f(path);
  if (!f.is_open()) {
    err = "cannot open " + path;
    return false;
  }
  std::string line;
  std::getline(f, line);
  if (!json_parse(line, out, err)) {
    err = path + ": " + err;
    return false;
  }
  return true;
}

}  // namespace fwigb
