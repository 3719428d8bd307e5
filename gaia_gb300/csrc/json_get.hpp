// JSON value access with the reference loader's EXTRACT_FROM_JSON semantics
// (a key that is present overrides the default, an absent key keeps it), plus
// small file helpers shared by the tet and cloth scene loaders.
#pragma once
#include <cstdint>
#include <fstream>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

#include "json_lite.hpp"

namespace gaia {
namespace jsonio {

inline std::string read_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::runtime_error("cannot open file: " + path);
    std::ostringstream ss;
    ss << f.rdbuf();
    return ss.str();
}

inline std::string replace_all(std::string s, const std::string& from, const std::string& to) {
    if (from.empty()) return s;
    size_t pos = 0;
    while ((pos = s.find(from, pos)) != std::string::npos) {
        s.replace(pos, from.size(), to);
        pos += to.size();
    }
    return s;
}

// EXTRACT_FROM_JSON semantics: read the key if present, keep the default otherwise.
inline void get(const json::Value& o, const char* k, double& out) {
    if (auto* v = o.find(k)) {
        if (v->type == json::Value::Number) out = v->num;
        else if (v->type == json::Value::Bool) out = v->b ? 1.0 : 0.0;
        else throw std::runtime_error(std::string("key '") + k + "' is not a number");
    }
}
inline void get(const json::Value& o, const char* k, int& out) {
    double d = out;
    get(o, k, d);
    out = int(d);
}
inline void get(const json::Value& o, const char* k, bool& out) {
    if (auto* v = o.find(k)) {
        if (v->type == json::Value::Bool) out = v->b;
        else if (v->type == json::Value::Number) out = v->num != 0.0;
        else throw std::runtime_error(std::string("key '") + k + "' is not a bool");
    }
}
inline void get(const json::Value& o, const char* k, std::string& out) {
    if (auto* v = o.find(k)) {
        if (v->type == json::Value::String) out = v->str;
        else throw std::runtime_error(std::string("key '") + k + "' is not a string");
    }
}
inline void get3(const json::Value& o, const char* k, double* out) {
    if (auto* v = o.find(k)) {
        if (!v->is_array() || v->arr.size() != 3) throw std::runtime_error(std::string("key '") + k + "' is not a 3-vector");
        for (int i = 0; i < 3; ++i) out[i] = v->arr[i].num;
    }
}
inline void get_ints(const json::Value& o, const char* k, std::vector<int32_t>& out) {
    if (auto* v = o.find(k)) {
        if (!v->is_array()) throw std::runtime_error(std::string("key '") + k + "' is not an array");
        out.clear();
        for (auto& e : v->arr) out.push_back(int32_t(e.num));
    }
}

}  // namespace jsonio
}  // namespace gaia
