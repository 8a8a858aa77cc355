// YAML reader for NNAP model files, into the same JValue tree as the JSON reader.
//
// The reference reads .yaml / .yml model files with Groovy's YamlSlurper (IO.yaml2map,
// IO.java:853; dispatch NNAP.java:407-411) and writes them with YamlBuilder.  This reader
// takes the subset such files use:
//   - block mappings "key: value" and block sequences "- item" by indentation, including a
//     sequence item that opens a mapping ("- key: value") or another sequence ("- - 0.1");
//   - flow sequences and mappings "[...]" / "{...}", which may span lines;
//   - plain, 'single' and "double" quoted scalars; numbers (with .inf / .nan), true /
//     false, null / ~; comments, "---" and "..." document markers.
// Anchors, aliases, tags, block scalars (| and >) and multi-line plain scalars are
// rejected with an error.
#pragma once

#include <cmath>
#include <cstdlib>
#include <cstring>
#include <limits>
#include <stdexcept>
#include <string>
#include <vector>

#include "json.hpp"

namespace nnapgb {

class YParser {
  public:
    YParser(const char* s, size_t n) { split(s, n); }

    JValue parse() {
        size_t i = 0;
        if (lines_.empty()) fail(0, "empty document");
        JValue v = node(i, lines_[0].indent);
        if (i != lines_.size()) fail(i, "unexpected content after the document");
        return v;
    }

  private:
    struct Line {
        int indent;
        std::string text;  // without indentation and comments; never empty
        int no;            // 1-based source line
    };
    std::vector<Line> lines_;

    [[noreturn]] void fail(size_t i, const std::string& m) const {
        const int no = i < lines_.size() ? lines_[i].no : (lines_.empty() ? 0 : lines_.back().no);
        throw std::runtime_error("YAML line " + std::to_string(no) + ": " + m);
    }

    // Drop a comment ("#" at the start or after a blank, outside quotes) and trailing blanks.
    static std::string strip(const std::string& s) {
        char q = 0;
        size_t end = s.size();
        for (size_t k = 0; k < s.size(); ++k) {
            const char c = s[k];
            if (q) {
                if (c == q) {
                    if (q == '\'' && k + 1 < s.size() && s[k + 1] == '\'') { ++k; continue; }
                    q = 0;
                } else if (q == '"' && c == '\\') {
                    ++k;
                }
            } else if (c == '"' || c == '\'') {
                if (k == 0 || s[k - 1] == ' ' || s[k - 1] == '[' || s[k - 1] == '{' || s[k - 1] == ',' ||
                    s[k - 1] == ':' || s[k - 1] == '-')
                    q = c;
            } else if (c == '#' && (k == 0 || s[k - 1] == ' ' || s[k - 1] == '\t')) {
                end = k;
                break;
            }
        }
        while (end > 0 && (s[end - 1] == ' ' || s[end - 1] == '\t' || s[end - 1] == '\r')) --end;
        return s.substr(0, end);
    }

    void split(const char* s, size_t n) {
        size_t a = 0;
        int no = 0;
        while (a <= n) {
            size_t b = a;
            while (b < n && s[b] != '\n') ++b;
            ++no;
            std::string raw(s + a, b - a);
            const size_t lead = raw.find_first_not_of(" \t");
            if (lead != std::string::npos && raw.find('\t') < lead)
                throw std::runtime_error("YAML line " + std::to_string(no) + ": tab indentation");
            std::string t = strip(raw);
            const size_t ind = t.find_first_not_of(' ');
            if (ind != std::string::npos) {
                std::string body = t.substr(ind);
                if (!(ind == 0 && (body == "---" || body == "..." || body.rfind("--- ", 0) == 0 || body[0] == '%'))) {
                    lines_.push_back({(int)ind, body, no});
                } else if (body.rfind("--- ", 0) == 0) {
                    lines_.push_back({0, body.substr(4), no});
                }
            }
            if (b >= n) break;
            a = b + 1;
        }
    }

    // Position of the ": " (or a final ":") that makes text a mapping entry, or npos.
    static size_t key_colon(const std::string& t) {
        char q = 0;
        int depth = 0;
        for (size_t k = 0; k < t.size(); ++k) {
            const char c = t[k];
            if (q) {
                if (c == q) q = 0;
                else if (q == '"' && c == '\\') ++k;
                continue;
            }
            if ((c == '"' || c == '\'') && k == 0) { q = c; continue; }
            if (c == '[' || c == '{') ++depth;
            else if (c == ']' || c == '}') --depth;
            else if (c == ':' && depth == 0 && (k + 1 == t.size() || t[k + 1] == ' ')) return k;
        }
        return std::string::npos;
    }

    static bool is_seq_item(const std::string& t) { return t == "-" || t.rfind("- ", 0) == 0; }

    // The node whose first line is lines_[i] at indentation ind.
    JValue node(size_t& i, int ind) {
        const Line& L = lines_[i];
        if (is_seq_item(L.text)) return sequence(i, ind);
        if (key_colon(L.text) != std::string::npos) return mapping(i, ind);
        // a scalar or flow value on its own line(s)
        std::string text = L.text;
        const int no = L.no;
        ++i;
        return value_text(text, i, no);
    }

    JValue sequence(size_t& i, int ind) {
        JValue v;
        v.kind = JValue::ARR;
        while (i < lines_.size() && lines_[i].indent == ind && is_seq_item(lines_[i].text)) {
            Line& L = lines_[i];
            if (L.text == "-") {  // the item is the block below
                ++i;
                if (i < lines_.size() && lines_[i].indent > ind) v.arr.push_back(node(i, lines_[i].indent));
                else v.arr.push_back(JValue());
                continue;
            }
            // "- rest": rest is the first line of the item, two columns further in
            size_t off = 2;
            while (off < L.text.size() && L.text[off] == ' ') ++off;
            L.indent = ind + (int)off;
            L.text = L.text.substr(off);
            v.arr.push_back(node(i, L.indent));
        }
        if (i < lines_.size() && lines_[i].indent > ind) fail(i, "bad indentation in a sequence");
        return v;
    }

    JValue mapping(size_t& i, int ind) {
        JValue v;
        v.kind = JValue::OBJ;
        while (i < lines_.size() && lines_[i].indent == ind && !is_seq_item(lines_[i].text)) {
            const Line L = lines_[i];
            const size_t c = key_colon(L.text);
            if (c == std::string::npos) fail(i, "expected 'key: value'");
            std::string key = scalar_text(L.text.substr(0, c), i);
            std::string rest = L.text.substr(c + 1);
            const size_t r0 = rest.find_first_not_of(' ');
            rest = r0 == std::string::npos ? std::string() : rest.substr(r0);
            ++i;
            JValue val;
            if (rest.empty()) {
                // block value: more indented lines, or a sequence at the same indentation
                if (i < lines_.size() && (lines_[i].indent > ind || (lines_[i].indent == ind && is_seq_item(lines_[i].text))))
                    val = node(i, lines_[i].indent);
            } else {
                if (rest[0] == '|' || rest[0] == '>') fail(i - 1, "block scalars are not supported");
                val = value_text(rest, i, L.no);
            }
            for (auto& kv : v.obj)
                if (kv.first == key) fail(i - 1, "duplicate key '" + key + "'");
            v.obj.emplace_back(std::move(key), std::move(val));
        }
        if (i < lines_.size() && lines_[i].indent > ind) fail(i, "bad indentation in a mapping");
        return v;
    }

    // A value given on a line: a flow collection (joined with following lines until its
    // brackets close) or a scalar.
    JValue value_text(std::string text, size_t& i, int no) {
        if (text[0] == '&' || text[0] == '*' || text[0] == '!') fail(i ? i - 1 : 0, "anchors, aliases and tags are not supported");
        if (text[0] == '[' || text[0] == '{') {
            while (!balanced(text)) {
                if (i >= lines_.size()) throw std::runtime_error("YAML line " + std::to_string(no) + ": unclosed flow collection");
                text += " " + lines_[i].text;
                ++i;
            }
            size_t p = 0;
            JValue v = flow(text, p, no);
            while (p < text.size() && text[p] == ' ') ++p;
            if (p != text.size()) throw std::runtime_error("YAML line " + std::to_string(no) + ": trailing text after a flow collection");
            return v;
        }
        // a plain scalar continued on more indented lines is not supported
        return scalar(text, no);
    }

    static bool balanced(const std::string& t) {
        int depth = 0;
        char q = 0;
        for (size_t k = 0; k < t.size(); ++k) {
            const char c = t[k];
            if (q) {
                if (c == q) q = 0;
                else if (q == '"' && c == '\\') ++k;
                continue;
            }
            if (c == '"' || c == '\'') q = c;
            else if (c == '[' || c == '{') ++depth;
            else if (c == ']' || c == '}') --depth;
        }
        return depth <= 0 && !q;
    }

    JValue flow(const std::string& t, size_t& p, int no) {
        auto ws = [&]() { while (p < t.size() && t[p] == ' ') ++p; };
        auto err = [&](const char* m) -> JValue { throw std::runtime_error("YAML line " + std::to_string(no) + ": " + m); };
        ws();
        if (p >= t.size()) return err("unexpected end of a flow collection");
        if (t[p] == '[') {
            JValue v;
            v.kind = JValue::ARR;
            ++p;
            ws();
            if (p < t.size() && t[p] == ']') { ++p; return v; }
            for (;;) {
                v.arr.push_back(flow(t, p, no));
                ws();
                if (p < t.size() && t[p] == ',') { ++p; ws(); if (p < t.size() && t[p] == ']') { ++p; return v; } continue; }
                if (p < t.size() && t[p] == ']') { ++p; return v; }
                return err("expected ',' or ']'");
            }
        }
        if (t[p] == '{') {
            JValue v;
            v.kind = JValue::OBJ;
            ++p;
            ws();
            if (p < t.size() && t[p] == '}') { ++p; return v; }
            for (;;) {
                ws();
                const size_t k0 = p;
                std::string key;
                if (t[p] == '"' || t[p] == '\'') {
                    key = quoted(t, p, no);
                } else {
                    while (p < t.size() && t[p] != ':' && t[p] != ',' && t[p] != '}') ++p;
                    key = trim(t.substr(k0, p - k0));
                }
                ws();
                if (p >= t.size() || t[p] != ':') return err("expected ':' in a flow mapping");
                ++p;
                JValue val = flow(t, p, no);
                v.obj.emplace_back(key, std::move(val));
                ws();
                if (p < t.size() && t[p] == ',') { ++p; continue; }
                if (p < t.size() && t[p] == '}') { ++p; return v; }
                return err("expected ',' or '}'");
            }
        }
        if (t[p] == '"' || t[p] == '\'') {
            JValue v;
            v.kind = JValue::STR;
            v.str = quoted(t, p, no);
            return v;
        }
        const size_t a = p;
        while (p < t.size() && t[p] != ',' && t[p] != ']' && t[p] != '}') ++p;
        return scalar(trim(t.substr(a, p - a)), no);
    }

    static std::string trim(const std::string& s) {
        const size_t a = s.find_first_not_of(' ');
        if (a == std::string::npos) return std::string();
        const size_t b = s.find_last_not_of(' ');
        return s.substr(a, b - a + 1);
    }

    static std::string quoted(const std::string& t, size_t& p, int no) {
        const char q = t[p++];
        std::string out;
        while (p < t.size()) {
            const char c = t[p++];
            if (c == q) {
                if (q == '\'' && p < t.size() && t[p] == '\'') { out += '\''; ++p; continue; }
                return out;
            }
            if (q == '"' && c == '\\' && p < t.size()) {
                const char e = t[p++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case '0': out += '\0'; break;
                    case '/': out += '/'; break;
                    case '"': out += '"'; break;
                    case '\\': out += '\\'; break;
                    case 'u': {
                        if (p + 4 > t.size()) throw std::runtime_error("YAML line " + std::to_string(no) + ": bad \\u escape");
                        const unsigned cp = (unsigned)std::strtoul(t.substr(p, 4).c_str(), nullptr, 16);
                        p += 4;
                        if (cp < 0x80) out += (char)cp;
                        else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                        else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                        break;
                    }
                    default: out += e;
                }
                continue;
            }
            out += c;
        }
        throw std::runtime_error("YAML line " + std::to_string(no) + ": unclosed quoted scalar");
    }

    std::string scalar_text(const std::string& s, size_t i) const {
        std::string t = trim(s);
        if (!t.empty() && (t[0] == '"' || t[0] == '\'')) {
            size_t p = 0;
            std::string out = quoted(t, p, i < lines_.size() ? lines_[i].no : 0);
            return out;
        }
        return t;
    }

    // Plain or quoted scalar, resolved as the YAML core schema does: null, booleans,
    // integers, floats (.inf, .nan), else a string.
    static JValue scalar(const std::string& s, int no) {
        JValue v;
        if (s.empty()) return v;
        if (s[0] == '"' || s[0] == '\'') {
            size_t p = 0;
            v.kind = JValue::STR;
            v.str = quoted(s, p, no);
            if (trim(s.substr(p)).size()) throw std::runtime_error("YAML line " + std::to_string(no) + ": text after a quoted scalar");
            return v;
        }
        if (s == "~" || s == "null" || s == "Null" || s == "NULL") return v;
        if (s == "true" || s == "True" || s == "TRUE") { v.kind = JValue::BOOL; v.b = true; return v; }
        if (s == "false" || s == "False" || s == "FALSE") { v.kind = JValue::BOOL; v.b = false; return v; }
        std::string u = s;
        int sign = 1;
        if (!u.empty() && (u[0] == '+' || u[0] == '-')) { sign = u[0] == '-' ? -1 : 1; u = u.substr(1); }
        if (u == ".inf" || u == ".Inf" || u == ".INF") {
            v.kind = JValue::NUM;
            v.num = sign * std::numeric_limits<double>::infinity();
            return v;
        }
        if (u == ".nan" || u == ".NaN" || u == ".NAN") {
            v.kind = JValue::NUM;
            v.num = std::numeric_limits<double>::quiet_NaN();
            return v;
        }
        // a number: digits, one optional '.', optional exponent (the whole text)
        bool num = !u.empty(), digit = false, dot = false, ex = false;
        for (size_t k = 0; k < u.size() && num; ++k) {
            const char c = u[k];
            if (c >= '0' && c <= '9') digit = true;
            else if (c == '.' && !dot && !ex) dot = true;
            else if ((c == 'e' || c == 'E') && digit && !ex) {
                ex = true;
                if (k + 1 < u.size() && (u[k + 1] == '+' || u[k + 1] == '-')) ++k;
                if (k + 1 >= u.size()) num = false;
            } else num = false;
        }
        if (num && digit) {
            v.kind = JValue::NUM;
            v.num = std::strtod(s.c_str(), nullptr);
            return v;
        }
        v.kind = JValue::STR;
        v.str = s;
        return v;
    }
};

}  // namespace nnapgb
