#include "json.h"

#include <cstdlib>
#include <cstring>

namespace illume {

const JValue* JValue::find(const char* key) const {
  if (type != Object) return nullptr;
  for (const auto& kv : obj)
    if (kv.first == key) return &kv.second;
  return nullptr;
}

namespace {

struct Parser {
  const char* s;
  size_t n, i = 0;
  std::string err;

  void ws() {
    while (i < n && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r')) ++i;
  }
  bool fail(const char* what) {
    if (err.empty()) err = std::string(what) + " at offset " + std::to_string(i);
    return false;
  }
  bool lit(const char* w) {
    const size_t L = strlen(w);
    if (i + L <= n && memcmp(s + i, w, L) == 0) { i += L; return true; }
    return false;
  }
  static void put_utf8(std::string& o, unsigned cp) {
    if (cp < 0x80) o += (char)cp;
    else if (cp < 0x800) { o += (char)(0xC0 | (cp >> 6)); o += (char)(0x80 | (cp & 0x3F)); }
    else if (cp < 0x10000) {
      o += (char)(0xE0 | (cp >> 12)); o += (char)(0x80 | ((cp >> 6) & 0x3F)); o += (char)(0x80 | (cp & 0x3F));
    } else {
      o += (char)(0xF0 | (cp >> 18)); o += (char)(0x80 | ((cp >> 12) & 0x3F));
      o += (char)(0x80 | ((cp >> 6) & 0x3F)); o += (char)(0x80 | (cp & 0x3F));
    }
  }
  bool hex4(unsigned* v) {
    if (i + 4 > n) return fail("truncated \\u escape");
    *v = 0;
    for (int k = 0; k < 4; ++k) {
      const char c = s[i++];
      *v <<= 4;
      if (c >= '0' && c <= '9') *v |= c - '0';
      else if (c >= 'a' && c <= 'f') *v |= c - 'a' + 10;
      else if (c >= 'A' && c <= 'F') *v |= c - 'A' + 10;
      else return fail("bad \\u escape");
    }
    return true;
  }
  bool string(std::string* o) {
    if (s[i] != '"') return fail("expected string");
    ++i;
    while (i < n && s[i] != '"') {
      const char c = s[i++];
      if ((unsigned char)c < 0x20) return fail("control character in string");
      if (c != '\\') { *o += c; continue; }
      if (i >= n) return fail("truncated escape");
      const char e = s[i++];
      switch (e) {
        case '"': *o += '"'; break;
        case '\\': *o += '\\'; break;
        case '/': *o += '/'; break;
        case 'b': *o += '\b'; break;
        case 'f': *o += '\f'; break;
        case 'n': *o += '\n'; break;
        case 'r': *o += '\r'; break;
        case 't': *o += '\t'; break;
        case 'u': {
          unsigned cp = 0;
          if (!hex4(&cp)) return false;
          if (cp >= 0xD800 && cp < 0xDC00 && i + 6 <= n && s[i] == '\\' && s[i + 1] == 'u') {
            i += 2;
            unsigned lo = 0;
            if (!hex4(&lo)) return false;
            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
          }
          put_utf8(*o, cp);
          break;
        }
        default: return fail("bad escape");
      }
    }
    if (i >= n) return fail("unterminated string");
    ++i;
    return true;
  }
  bool number(JValue* v) {
    const size_t st = i;
    if (s[i] == '-') ++i;
    if (i >= n || !(s[i] >= '0' && s[i] <= '9')) return fail("bad number");
    while (i < n && s[i] >= '0' && s[i] <= '9') ++i;
    bool integer = true;
    if (i < n && s[i] == '.') {
      integer = false;
      ++i;
      if (i >= n || !(s[i] >= '0' && s[i] <= '9')) return fail("bad fraction");
      while (i < n && s[i] >= '0' && s[i] <= '9') ++i;
    }
    if (i < n && (s[i] == 'e' || s[i] == 'E')) {
      integer = false;
      ++i;
      if (i < n && (s[i] == '+' || s[i] == '-')) ++i;
      if (i >= n || !(s[i] >= '0' && s[i] <= '9')) return fail("bad exponent");
      while (i < n && s[i] >= '0' && s[i] <= '9') ++i;
    }
    std::string tok(s + st, i - st);
    v->type = JValue::Number;
    v->num = strtod(tok.c_str(), nullptr);
    v->is_integer = integer;
    return true;
  }
  bool value(JValue* v, int depth) {
    if (depth > 256) return fail("nesting too deep");
    ws();
    if (i >= n) return fail("unexpected end");
    const char c = s[i];
    if (c == '{') {
      ++i;
      v->type = JValue::Object;
      ws();
      if (i < n && s[i] == '}') { ++i; return true; }
      for (;;) {
        ws();
        std::string key;
        if (i >= n || !string(&key)) return fail("expected key");
        ws();
        if (i >= n || s[i] != ':') return fail("expected ':'");
        ++i;
        JValue child;
        if (!value(&child, depth + 1)) return false;
        v->obj.emplace_back(std::move(key), std::move(child));
        ws();
        if (i < n && s[i] == ',') { ++i; continue; }
        if (i < n && s[i] == '}') { ++i; return true; }
        return fail("expected ',' or '}'");
      }
    }
    if (c == '[') {
      ++i;
      v->type = JValue::Array;
      ws();
      if (i < n && s[i] == ']') { ++i; return true; }
      for (;;) {
        JValue child;
        if (!value(&child, depth + 1)) return false;
        v->arr.push_back(std::move(child));
        ws();
        if (i < n && s[i] == ',') { ++i; continue; }
        if (i < n && s[i] == ']') { ++i; return true; }
        return fail("expected ',' or ']'");
      }
    }
    if (c == '"') { v->type = JValue::String; return string(&v->str); }
    if (lit("true")) { v->type = JValue::Bool; v->b = true; return true; }
    if (lit("false")) { v->type = JValue::Bool; v->b = false; return true; }
    if (lit("null")) { v->type = JValue::Null; return true; }
    return number(v);
  }
};

}  // namespace

bool json_parse(const std::string& text, JValue* out, std::string* err) {
  Parser p{text.data(), text.size()};
  *out = JValue();
  if (!p.value(out, 0)) { if (err) *err = p.err; return false; }
  p.ws();
  if (p.i != p.n) { if (err) *err = "trailing characters at offset " + std::to_string(p.i); return false; }
  return true;
}

}  // namespace illume
