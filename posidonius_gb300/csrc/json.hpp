// json.hpp -- minimal JSON DOM for Posidonius case files.
//
// Numbers keep their source text and are converted with strtod (correctly
// rounded, as serde_json's reader), object members keep their order.
#pragma once
#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace posi {
namespace json {

struct Value {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    std::string text;  // number literal or string contents
    std::vector<Value> items;
    std::vector<std::pair<std::string, Value>> members;

    bool is_object() const { return kind == Object; }
    bool is_array() const { return kind == Array; }
    bool is_string() const { return kind == String; }
    bool is_number() const { return kind == Number; }

    const Value* find(const char* key) const {
        if (kind != Object) return nullptr;
        for (const auto& m : members)
            if (m.first == key) return &m.second;
        return nullptr;
    }
    double num() const { return kind == Number ? std::strtod(text.c_str(), nullptr) : 0.0; }
    int64_t integer() const { return kind == Number ? (int64_t)std::strtoll(text.c_str(), nullptr, 10) : 0; }
};

class Parser {
public:
    Parser(const char* s, size_t n) : p_(s), e_(s + n) {}

    bool parse(Value& out, std::string& err) {
        ws();
        if (!value(out, 0)) { err = err_.empty() ? "syntax error" : err_; return false; }
        ws();
        if (p_ != e_) { err = "trailing characters"; return false; }
        return true;
    }

private:
    const char* p_;
    const char* e_;
    std::string err_;

    void ws() {
        while (p_ < e_ && (*p_ == ' ' || *p_ == '\n' || *p_ == '\r' || *p_ == '\t')) ++p_;
    }
    bool lit(const char* w) {
        size_t n = std::strlen(w);
        if ((size_t)(e_ - p_) < n || std::strncmp(p_, w, n) != 0) return false;
        p_ += n;
        return true;
    }
    bool string(std::string& out) {
        if (p_ >= e_ || *p_ != '"') return false;
        ++p_;
        out.clear();
        while (p_ < e_ && *p_ != '"') {
            char c = *p_++;
            if (c == '\\') {
                if (p_ >= e_) return false;
                char x = *p_++;
                switch (x) {
                    case '"': out += '"'; break;
                    case '\\': out += '\\'; break;
                    case '/': out += '/'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'n': out += '\n'; break;
                    case 'r': out += '\r'; break;
                    case 't': out += '\t'; break;
                    case 'u': {
                        if (e_ - p_ < 4) return false;
                        unsigned cp = (unsigned)std::strtoul(std::string(p_, 4).c_str(), nullptr, 16);
                        p_ += 4;
                        if (cp < 0x80) out += (char)cp;
                        else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                        else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                        break;
                    }
                    default: return false;
                }
            } else {
                out += c;
            }
        }
        if (p_ >= e_) return false;
        ++p_;
        return true;
    }
    bool number(Value& v) {
        const char* s = p_;
        if (p_ < e_ && (*p_ == '-' || *p_ == '+')) ++p_;
        bool digits = false;
        while (p_ < e_ && ((*p_ >= '0' && *p_ <= '9') || *p_ == '.' || *p_ == 'e' || *p_ == 'E' || *p_ == '-' || *p_ == '+')) {
            digits = true;
            ++p_;
        }
        if (!digits) return false;
        v.kind = Value::Number;
        v.text.assign(s, p_);
        char* end = nullptr;
        std::strtod(v.text.c_str(), &end);
        return end && *end == '\0';
    }
    bool value(Value& v, int depth) {
        if (depth > 64) { err_ = "nesting too deep"; return false; }
        ws();
        if (p_ >= e_) return false;
        char c = *p_;
        if (c == '{') {
            ++p_;
            v.kind = Value::Object;
            ws();
            if (p_ < e_ && *p_ == '}') { ++p_; return true; }
            for (;;) {
                ws();
                std::string key;
                if (!string(key)) return false;
                ws();
                if (p_ >= e_ || *p_ != ':') return false;
                ++p_;
                v.members.emplace_back(std::move(key), Value());
                if (!value(v.members.back().second, depth + 1)) return false;
                ws();
                if (p_ < e_ && *p_ == ',') { ++p_; continue; }
                if (p_ < e_ && *p_ == '}') { ++p_; return true; }
                return false;
            }
        }
        if (c == '[') {
            ++p_;
            v.kind = Value::Array;
            ws();
            if (p_ < e_ && *p_ == ']') { ++p_; return true; }
            for (;;) {
                v.items.emplace_back();
                if (!value(v.items.back(), depth + 1)) return false;
                ws();
                if (p_ < e_ && *p_ == ',') { ++p_; continue; }
                if (p_ < e_ && *p_ == ']') { ++p_; return true; }
                return false;
            }
        }
        if (c == '"') { v.kind = Value::String; return string(v.text); }
        if (lit("true")) { v.kind = Value::Bool; v.b = true; return true; }
        if (lit("false")) { v.kind = Value::Bool; v.b = false; return true; }
        if (lit("null")) { v.kind = Value::Null; return true; }
        return number(v);
    }
};

}  // namespace json
}  // namespace posi
