// Minimal JSON reader for the FwiFlow parameter and survey files.
//
// The reference reads the first line of each file with rapidjson
// (Parameter.cpp:27-33, Src_Rec.cu:24-35); this is a small recursive-descent
// parser of standard JSON (objects, arrays, strings, numbers, literals) that
// reports errors instead of asserting.
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

namespace fwigb {

struct JValue {
  enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
  bool b = false;
  double num = 0.0;
  bool is_integer = false;  // number written without fraction or exponent
  std::string str;
  std::vector<JValue> arr;
  std::map<std::string, JValue> obj;

  const JValue* get(const std::string& key) const {
    if (kind != Object) return nullptr;
    auto it = obj.find(key);
    return it == obj.end() ? nullptr : &it->second;
  }
};

// Parses `text`; on failure returns false and sets `err`.
bool json_parse(const std::string& text, JValue& out, std::string& err);

// Reads the first line of a file (the reference's convention) and parses it.
bool json_read_first_line(const std::string& path, JValue& out, std::string& err);

}  // namespace fwigb
