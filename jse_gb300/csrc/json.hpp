// Minimal JSON reader for NNAP model files (objects, arrays, numbers, strings,
// booleans, null).  Numbers are parsed with strtod so FP64 model values are exact.
#pragma once

#include <algorithm>
#include <cctype>
#include <cstdlib>
#include <limits>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace nnapgb {

struct JValue {
    enum Kind { NUL, BOOL, NUM, STR, ARR, OBJ } kind = NUL;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<JValue> arr;
    std::vector<std::pair<std::string, JValue>> obj;

    const JValue* get(const std::string& k) const {
        if (kind != OBJ) return nullptr;
        for (auto& kv : obj)
            if (kv.first == k) return kv.second.kind == NUL ? nullptr : &kv.second;
        return nullptr;
    }
    // First non-null of several keys (UT.Code.get semantics).
    const JValue* get_any(std::initializer_list<const char*> ks) const {
        for (const char* k : ks)
            if (const JValue* v = get(k)) return v;
        return nullptr;
    }
    double as_num() const {
        if (kind != NUM) throw std::runtime_error("expected a number");
        return num;
    }
    int as_int() const { return (int)as_num(); }
    const std::string& as_str() const {
        if (kind != STR) throw std::runtime_error("expected a string");
        return str;
    }
};

class JParser {
  public:
    JParser(const char* s, size_t n) : p_(s), e_(s + n) {}
    JValue parse() {
        JValue v = value();
        ws();
        if (p_ != e_) throw std::runtime_error("trailing characters after JSON value");
        return v;
    }

  private:
    const char* p_;
    const char* e_;
    void ws() {
        while (p_ < e_ && (*p_ == ' ' || *p_ == '\n' || *p_ == '\t' || *p_ == '\r')) ++p_;
    }
    [[noreturn]] void fail(const char* m) { throw std::runtime_error(std::string("JSON: ") + m); }
    bool lit(const char* w) {
        size_t n = std::char_traits<char>::length(w);
        if ((size_t)(e_ - p_) >= n && std::equal(w, w + n, p_)) { p_ += n; return true; }
        return false;
    }
    JValue value() {
        ws();
        if (p_ >= e_) fail("unexpected end");
        JValue v;
        char c = *p_;
        if (c == '{') {
            v.kind = JValue::OBJ;
            ++p_;
            ws();
            if (p_ < e_ && *p_ == '}') { ++p_; return v; }
            for (;;) {
                ws();
                if (p_ >= e_ || *p_ != '"') fail("expected key");
                std::string k = string();
                ws();
                if (p_ >= e_ || *p_ != ':') fail("expected ':'");
                ++p_;
                v.obj.emplace_back(std::move(k), value());
                ws();
                if (p_ < e_ && *p_ == ',') { ++p_; continue; }
                if (p_ < e_ && *p_ == '}') { ++p_; return v; }
                fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            v.kind = JValue::ARR;
            ++p_;
            ws();
            if (p_ < e_ && *p_ == ']') { ++p_; return v; }
            for (;;) {
                v.arr.push_back(value());
                ws();
                if (p_ < e_ && *p_ == ',') { ++p_; continue; }
                if (p_ < e_ && *p_ == ']') { ++p_; return v; }
                fail("expected ',' or ']'");
            }
        }
        if (c == '"') { v.kind = JValue::STR; v.str = string(); return v; }
        if (lit("true")) { v.kind = JValue::BOOL; v.b = true; return v; }
        if (lit("false")) { v.kind = JValue::BOOL; v.b = false; return v; }
        if (lit("null")) return v;
        if (lit("NaN")) { v.kind = JValue::NUM; v.num = std::numeric_limits<double>::quiet_NaN(); return v; }
        std::string buf;
        while (p_ < e_ && (std::isdigit((unsigned char)*p_) || *p_ == '-' || *p_ == '+' || *p_ == '.' ||
                           *p_ == 'e' || *p_ == 'E'))
            buf.push_back(*p_++);
        if (buf.empty()) fail("unexpected character");
        char* end = nullptr;
        v.kind = JValue::NUM;
        v.num = std::strtod(buf.c_str(), &end);
        if (!end || *end) fail("bad number");
        return v;
    }
    std::string string() {
        ++p_;  // opening quote
        std::string s;
        while (p_ < e_ && *p_ != '"') {
            char c = *p_++;
            if (c == '\\') {
                if (p_ >= e_) fail("bad escape");
                char x = *p_++;
                switch (x) {
                    case 'n': s.push_back('\n'); break;
                    case 't': s.push_back('\t'); break;
                    case 'r': s.push_back('\r'); break;
                    case 'b': s.push_back('\b'); break;
                    case 'f': s.push_back('\f'); break;
                    case 'u': {
                        if (e_ - p_ < 4) fail("bad unicode escape");
                        unsigned cp = (unsigned)std::strtoul(std::string(p_, p_ + 4).c_str(), nullptr, 16);
                        p_ += 4;
                        if (cp < 0x80) s.push_back((char)cp);
                        else if (cp < 0x800) { s.push_back((char)(0xC0 | (cp >> 6))); s.push_back((char)(0x80 | (cp & 0x3F))); }
                        else { s.push_back((char)(0xE0 | (cp >> 12))); s.push_back((char)(0x80 | ((cp >> 6) & 0x3F))); s.push_back((char)(0x80 | (cp & 0x3F))); }
                        break;
                    }
                    default: s.push_back(x);
                }
            } else {
                s.push_back(c);
            }
        }
        if (p_ >= e_) fail("unterminated string");
        ++p_;
        return s;
    }
};

}  // namespace nnapgb
