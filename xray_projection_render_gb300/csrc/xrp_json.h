// xrp_json.h -- a small JSON reader for the scene and deformation maps.
//
// The library takes the reference's object and deformation schema as JSON
// text, the form the reference itself writes (object.json, main.go:536-546)
// and reads (main.go:90-120).  Numbers are kept as doubles with a flag telling
// whether the literal was integral, so the loader can reproduce the
// reference's int-versus-float type checks where they matter.
#pragma once
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace xrp {

struct JValue {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    bool integral = false;
    std::string str;
    std::vector<JValue> arr;
    std::vector<std::pair<std::string, JValue>> obj;

    const JValue* get(const std::string& key) const {
        if (kind != Object) return nullptr;
        for (auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    bool is_num() const { return kind == Number; }
};

class JsonError : public std::runtime_error {
  public:
    using std::runtime_error::runtime_error;
};

class JsonParser {
  public:
    explicit JsonParser(const char* text) : p_(text), start_(text) {}

    JValue parse() {
        JValue v = value();
        ws();
        if (*p_) fail("trailing characters");
        return v;
    }

  private:
    const char* p_;
    const char* start_;
    int depth_ = 0;

    [[noreturn]] void fail(const char* what) {
        throw JsonError(std::string("JSON: ") + what + " at offset " + std::to_string(p_ - start_));
    }
    void ws() {
        while (*p_ == ' ' || *p_ == '\n' || *p_ == '\r' || *p_ == '\t') p_++;
    }
    JValue value() {
        ws();
        if (++depth_ > 64) fail("nesting too deep");
        JValue v;
        switch (*p_) {
        case '{': v = object(); break;
        case '[': v = array(); break;
        case '"': v.kind = JValue::String; v.str = string(); break;
        case 't': lit("true"); v.kind = JValue::Bool; v.b = true; break;
        case 'f': lit("false"); v.kind = JValue::Bool; v.b = false; break;
        case 'n': lit("null"); v.kind = JValue::Null; break;
        default: v = number(); break;
        }
        depth_--;
        return v;
    }
    void lit(const char* s) {
        size_t n = strlen(s);
        if (strncmp(p_, s, n) != 0) fail("bad literal");
        p_ += n;
    }
    JValue number() {
        const char* s = p_;
        if (*p_ == '-') p_++;
        if (!(*p_ >= '0' && *p_ <= '9')) fail("bad value");
        bool integral = true;
        while ((*p_ >= '0' && *p_ <= '9')) p_++;
        if (*p_ == '.') {
            integral = false;
            p_++;
            while (*p_ >= '0' && *p_ <= '9') p_++;
        }
        if (*p_ == 'e' || *p_ == 'E') {
            integral = false;
            p_++;
            if (*p_ == '+' || *p_ == '-') p_++;
            while (*p_ >= '0' && *p_ <= '9') p_++;
        }
        JValue v;
        v.kind = JValue::Number;
        v.num = strtod(std::string(s, p_).c_str(), nullptr);
        v.integral = integral;
        return v;
    }
    std::string string() {
        if (*p_ != '"') fail("expected string");
        p_++;
        std::string out;
        while (*p_ && *p_ != '"') {
            if (*p_ == '\\') {
                p_++;
                switch (*p_) {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    unsigned cp = 0;
                    for (int k = 1; k <= 4; k++) {
                        char c = p_[k];
                        cp <<= 4;
                        if (c >= '0' && c <= '9') cp |= (unsigned)(c - '0');
                        else if (c >= 'a' && c <= 'f') cp |= (unsigned)(c - 'a' + 10);
                        else if (c >= 'A' && c <= 'F') cp |= (unsigned)(c - 'A' + 10);
                        else fail("bad \\u escape");
                    }
                    p_ += 4;
                    if (cp < 0x80) out += (char)cp;
                    else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                    else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                    break;
                }
                default: fail("bad escape");
                }
                p_++;
            } else {
                out += *p_++;
            }
        }
        if (*p_ != '"') fail("unterminated string");
        p_++;
        return out;
    }
    JValue array() {
        JValue v;
        v.kind = JValue::Array;
        p_++;
        ws();
        if (*p_ == ']') { p_++; return v; }
        for (;;) {
            v.arr.push_back(value());
            ws();
            if (*p_ == ',') { p_++; continue; }
            if (*p_ == ']') { p_++; return v; }
            fail("expected , or ]");
        }
    }
    JValue object() {
        JValue v;
        v.kind = JValue::Object;
        p_++;
        ws();
        if (*p_ == '}') { p_++; return v; }
        for (;;) {
            ws();
            std::string k = string();
            ws();
            if (*p_ != ':') fail("expected :");
            p_++;
            JValue val = value();
            bool replaced = false;
            for (auto& kv : v.obj)
                if (kv.first == k) { kv.second = val; replaced = true; }
            if (!replaced) v.obj.emplace_back(k, std::move(val));
            ws();
            if (*p_ == ',') { p_++; continue; }
            if (*p_ == '}') { p_++; return v; }
            fail("expected , or }");
        }
    }
};

inline JValue parse_json(const char* text) { return JsonParser(text).parse(); }

}  // namespace xrp
