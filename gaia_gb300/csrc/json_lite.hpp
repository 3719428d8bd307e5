// Minimal JSON reader for Models.json / Parameters.json / coloring files.
// Supports the full JSON grammar (objects, arrays, numbers, strings with
// escapes, true/false/null); numbers are kept as double. Errors throw
// std::runtime_error with the byte offset.
#pragma once
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace gaia {
namespace json {

struct Value {
    enum Type { Null, Bool, Number, String, Array, Object } type = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Value> arr;
    std::vector<std::pair<std::string, Value>> obj;  // insertion order kept

    const Value* find(const std::string& key) const {
        if (type != Object) return nullptr;
        for (auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    bool is_number() const { return type == Number; }
    bool is_array() const { return type == Array; }
    bool is_object() const { return type == Object; }
};

class Parser {
public:
    Parser(const char* s, size_t n) : s_(s), n_(n) {}
    Value parse() {
        Value v = value();
        ws();
        if (i_ != n_) fail("trailing characters");
        return v;
    }

private:
    const char* s_;
    size_t n_, i_ = 0;
    [[noreturn]] void fail(const char* what) {
        throw std::runtime_error(std::string("json: ") + what + " at byte " + std::to_string(i_));
    }
    void ws() {
        while (i_ < n_ && (s_[i_] == ' ' || s_[i_] == '\n' || s_[i_] == '\r' || s_[i_] == '\t')) ++i_;
    }
    bool lit(const char* w) {
        size_t k = std::strlen(w);
        if (i_ + k <= n_ && std::strncmp(s_ + i_, w, k) == 0) {
            i_ += k;
            return true;
        }
        return false;
    }
    Value value() {
        ws();
        if (i_ >= n_) fail("unexpected end");
        char c = s_[i_];
        Value v;
        if (c == '{') {
            v.type = Value::Object;
            ++i_;
            ws();
            if (i_ < n_ && s_[i_] == '}') { ++i_; return v; }
            for (;;) {
                ws();
                if (i_ >= n_ || s_[i_] != '"') fail("expected key");
                std::string k = string();
                ws();
                if (i_ >= n_ || s_[i_] != ':') fail("expected ':'");
                ++i_;
                v.obj.emplace_back(std::move(k), value());
                ws();
                if (i_ < n_ && s_[i_] == ',') { ++i_; continue; }
                if (i_ < n_ && s_[i_] == '}') { ++i_; break; }
                fail("expected ',' or '}'");
            }
        } else if (c == '[') {
            v.type = Value::Array;
            ++i_;
            ws();
            if (i_ < n_ && s_[i_] == ']') { ++i_; return v; }
            for (;;) {
                v.arr.push_back(value());
                ws();
                if (i_ < n_ && s_[i_] == ',') { ++i_; continue; }
                if (i_ < n_ && s_[i_] == ']') { ++i_; break; }
                fail("expected ',' or ']'");
            }
        } else if (c == '"') {
            v.type = Value::String;
            v.str = string();
        } else if (lit("true")) {
            v.type = Value::Bool; v.b = true;
        } else if (lit("false")) {
            v.type = Value::Bool; v.b = false;
        } else if (lit("null")) {
            v.type = Value::Null;
        } else if (c == '-' || (c >= '0' && c <= '9')) {
            const char* b = s_ + i_;
            char* e = nullptr;
            v.type = Value::Number;
            v.num = std::strtod(b, &e);
            if (e == b) fail("bad number");
            i_ += size_t(e - b);
        } else if (lit("NaN")) {
            v.type = Value::Number; v.num = std::strtod("nan", nullptr);
        } else {
            fail("unexpected character");
        }
        return v;
    }
    std::string string() {
        ++i_;  // opening quote
        std::string out;
        while (i_ < n_) {
            char c = s_[i_++];
            if (c == '"') return out;
            if (c != '\\') { out.push_back(c); continue; }
            if (i_ >= n_) fail("bad escape");
            char e = s_[i_++];
            switch (e) {
                case '"': out.push_back('"'); break;
                case '\\': out.push_back('\\'); break;
                case '/': out.push_back('/'); break;
                case 'b': out.push_back('\b'); break;
                case 'f': out.push_back('\f'); break;
                case 'n': out.push_back('\n'); break;
                case 'r': out.push_back('\r'); break;
                case 't': out.push_back('\t'); break;
                case 'u': {
                    if (i_ + 4 > n_) fail("bad \\u escape");
                    unsigned cp = unsigned(std::strtoul(std::string(s_ + i_, 4).c_str(), nullptr, 16));
                    i_ += 4;
                    if (cp < 0x80) out.push_back(char(cp));
                    else if (cp < 0x800) { out.push_back(char(0xC0 | (cp >> 6))); out.push_back(char(0x80 | (cp & 0x3F))); }
                    else { out.push_back(char(0xE0 | (cp >> 12))); out.push_back(char(0x80 | ((cp >> 6) & 0x3F))); out.push_back(char(0x80 | (cp & 0x3F))); }
                    break;
                }
                default: fail("bad escape");
            }
        }
        fail("unterminated string");
    }
};

inline Value parse(const std::string& text) { return Parser(text.data(), text.size()).parse(); }

}  // namespace json
}  // namespace gaia
