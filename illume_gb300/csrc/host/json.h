// Minimal JSON DOM for the reference's scene format (RFC 8259 values; numbers kept as
// double and read as float the way the reference's rapidjson GetFloat does).
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

namespace illume {

struct JValue {
  enum Type { Null, Bool, Number, String, Array, Object } type = Null;
  bool b = false;
  double num = 0.0;
  bool is_integer = false;  // written without fraction or exponent
  std::string str;
  std::vector<JValue> arr;
  std::vector<std::pair<std::string, JValue>> obj;

  const JValue* find(const char* key) const;
  bool is_number() const { return type == Number; }
  bool is_array() const { return type == Array; }
  bool is_object() const { return type == Object; }
  bool is_string() const { return type == String; }
  float as_float() const { return (float)num; }
  int as_int() const { return (int)num; }
};

// Parses text; on failure returns false and sets *err (with the byte offset).
bool json_parse(const std::string& text, JValue* out, std::string* err);

}  // namespace illume
