// Minimal JSON reader for case files.
//
// The reference reads its case files with nlohmann/json 3.7.0, whose lexer hands
// every floating-point token to strtod; this reader does the same, so a decimal in a
// case file becomes the same double on both sides.  Integers are kept as doubles
// too (every integer a case file holds is far below 2^53).
#pragma once

#include <cctype>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace hf {

struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    bool has(const std::string& k) const { return kind == Object && obj.count(k) != 0; }
    const Json& operator[](const std::string& k) const {
        auto it = obj.find(k);
        if (kind != Object || it == obj.end()) throw std::runtime_error("missing key '" + k + "'");
        return it->second;
    }
    const Json& operator[](size_t i) const {
        if (kind != Array || i >= arr.size()) throw std::runtime_error("bad array index");
        return arr[i];
    }
    size_t size() const { return kind == Array ? arr.size() : (kind == Object ? obj.size() : 0); }
    double number() const {
        if (kind != Number) throw std::runtime_error("expected a number");
        return num;
    }
    const std::string& string() const {
        if (kind != String) throw std::runtime_error("expected a string");
        return str;
    }

    static Json parse(const char* s, size_t n) {
        Parser p{s, s + n};
        Json v = p.value();
        p.ws();
        if (p.p != p.e) throw std::runtime_error("trailing characters in JSON");
        return v;
    }

  private:
    struct Parser {
        const char* p;
        const char* e;
        void ws() {
            while (p < e && (*p == ' ' || *p == '\n' || *p == '\r' || *p == '\t')) ++p;
        }
        [[noreturn]] void fail(const char* what) { throw std::runtime_error(what); }
        Json value() {
            ws();
            if (p >= e) fail("unexpected end of JSON");
            Json v;
            char c = *p;
            if (c == '{') {
                v.kind = Object;
                ++p;
                ws();
                if (p < e && *p == '}') { ++p; return v; }
                for (;;) {
                    ws();
                    Json k = value();
                    if (k.kind != String) fail("object key must be a string");
                    ws();
                    if (p >= e || *p != ':') fail("expected ':'");
                    ++p;
                    v.obj[k.str] = value();
                    ws();
                    if (p < e && *p == ',') { ++p; continue; }
                    if (p < e && *p == '}') { ++p; return v; }
                    fail("expected ',' or '}'");
                }
            }
            if (c == '[') {
                v.kind = Array;
                ++p;
                ws();
                if (p < e && *p == ']') { ++p; return v; }
                for (;;) {
                    v.arr.push_back(value());
                    ws();
                    if (p < e && *p == ',') { ++p; continue; }
                    if (p < e && *p == ']') { ++p; return v; }
                    fail("expected ',' or ']'");
                }
            }
            if (c == '"') {
                v.kind = String;
                ++p;
                while (p < e && *p != '"') {
                    if (*p == '\\') {
                        ++p;
                        if (p >= e) fail("bad escape");
                        char x = *p;
                        v.str.push_back(x == 'n' ? '\n' : x == 't' ? '\t' : x);
                    } else {
                        v.str.push_back(*p);
                    }
                    ++p;
                }
                if (p >= e) fail("unterminated string");
                ++p;
                return v;
            }
            if (c == 't' && e - p >= 4 && std::string(p, 4) == "true") { v.kind = Bool; v.b = true; p += 4; return v; }
            if (c == 'f' && e - p >= 5 && std::string(p, 5) == "false") { v.kind = Bool; p += 5; return v; }
            if (c == 'n' && e - p >= 4 && std::string(p, 4) == "null") { p += 4; return v; }
            // number: collect the token, convert with strtod
            const char* s = p;
            while (p < e && (std::isdigit((unsigned char)*p) || *p == '-' || *p == '+' || *p == '.' ||
                             *p == 'e' || *p == 'E'))
                ++p;
            if (s == p) fail("unexpected character in JSON");
            std::string tok(s, p);
            char* end = nullptr;
            v.kind = Number;
            v.num = std::strtod(tok.c_str(), &end);
            if (end == tok.c_str() || *end != '\0') fail("bad number");
            return v;
        }
    };
};

}  // namespace hf
