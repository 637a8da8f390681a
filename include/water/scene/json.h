// A small JSON reader for scene files (RFC 8259 values: null, booleans,
// numbers, strings with escapes, arrays, objects). Parse errors throw
// water::scene::JsonError with the byte offset. Only what load_scene needs is
// exposed: typed getters that throw on a type mismatch.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace water::scene {

struct JsonError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

class Json {
public:
    enum class Type { Null, Bool, Number, String, Array, Object };

    Json() = default;
    Type type() const noexcept { return type_; }
    bool is_object() const noexcept { return type_ == Type::Object; }
    bool is_array() const noexcept { return type_ == Type::Array; }
    bool is_number() const noexcept { return type_ == Type::Number; }
    bool is_string() const noexcept { return type_ == Type::String; }

    bool contains(const std::string& key) const { return type_ == Type::Object && obj_.count(key) != 0; }
    const Json& at(const std::string& key) const {
        if (type_ != Type::Object) throw JsonError("JSON: not an object (looking for \"" + key + "\")");
        auto it = obj_.find(key);
        if (it == obj_.end()) throw JsonError("JSON: missing key \"" + key + "\"");
        return it->second;
    }
    const Json& operator[](const std::string& key) const { return at(key); }
    const Json& at(std::size_t i) const {
        if (type_ != Type::Array) throw JsonError("JSON: not an array");
        if (i >= arr_.size()) throw JsonError("JSON: index out of range");
        return arr_[i];
    }
    const Json& operator[](std::size_t i) const { return at(i); }
    const Json& operator[](int i) const { return at(static_cast<std::size_t>(i)); }
    std::size_t size() const noexcept { return type_ == Type::Array ? arr_.size() : obj_.size(); }

    double as_number() const {
        if (type_ != Type::Number) throw JsonError("JSON: value is not a number");
        return num_;
    }
    float as_float() const { return static_cast<float>(as_number()); }
    int as_int() const {
        const double v = as_number();
        if (v != static_cast<double>(static_cast<long long>(v))) throw JsonError("JSON: value is not an integer");
        return static_cast<int>(v);
    }
    bool as_bool() const {
        if (type_ != Type::Bool) throw JsonError("JSON: value is not a boolean");
        return b_;
    }
    const std::string& as_string() const {
        if (type_ != Type::String) throw JsonError("JSON: value is not a string");
        return str_;
    }

    static Json parse(const std::string& text) {
        Parser p{text, 0};
        p.ws();
        Json v = p.value(0);
        p.ws();
        if (p.i != text.size()) p.fail("trailing characters");
        return v;
    }

private:
    Type type_ = Type::Null;
    bool b_ = false;
    double num_ = 0.0;
    std::string str_;
    std::vector<Json> arr_;
    std::map<std::string, Json> obj_;

    struct Parser {
        const std::string& s;
        std::size_t i;

        [[noreturn]] void fail(const char* what) const {
            throw JsonError(std::string("JSON parse error at byte ") + std::to_string(i) + ": " + what);
        }
        void ws() {
            while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r')) ++i;
        }
        bool eat(char c) {
            ws();
            if (i < s.size() && s[i] == c) { ++i; return true; }
            return false;
        }
        void expect(char c) {
            if (!eat(c)) fail((std::string("expected '") + c + "'").c_str());
        }
        bool lit(const char* w) {
            std::size_t n = 0;
            while (w[n]) ++n;
            if (s.compare(i, n, w) == 0) { i += n; return true; }
            return false;
        }
        Json value(int depth) {
            if (depth > 256) fail("nesting too deep");
            ws();
            if (i >= s.size()) fail("unexpected end");
            Json v;
            const char c = s[i];
            if (c == '{') {
                ++i;
                v.type_ = Type::Object;
                if (eat('}')) return v;
                do {
                    ws();
                    if (i >= s.size() || s[i] != '"') fail("expected a key string");
                    std::string k = string();
                    expect(':');
                    v.obj_[k] = value(depth + 1);
                } while (eat(','));
                expect('}');
            } else if (c == '[') {
                ++i;
                v.type_ = Type::Array;
                if (eat(']')) return v;
                do {
                    v.arr_.push_back(value(depth + 1));
                } while (eat(','));
                expect(']');
            } else if (c == '"') {
                v.type_ = Type::String;
                v.str_ = string();
            } else if (lit("true")) {
                v.type_ = Type::Bool; v.b_ = true;
            } else if (lit("false")) {
                v.type_ = Type::Bool; v.b_ = false;
            } else if (lit("null")) {
                v.type_ = Type::Null;
            } else if (c == '-' || (c >= '0' && c <= '9')) {
                v.type_ = Type::Number;
                v.num_ = number();
            } else {
                fail("unexpected character");
            }
            return v;
        }
        double number() {
            const std::size_t start = i;
            if (s[i] == '-') ++i;
            if (i >= s.size() || !(s[i] >= '0' && s[i] <= '9')) fail("bad number");
            if (s[i] == '0') ++i;
            else while (i < s.size() && s[i] >= '0' && s[i] <= '9') ++i;
            if (i < s.size() && s[i] == '.') {
                ++i;
                if (i >= s.size() || !(s[i] >= '0' && s[i] <= '9')) fail("bad fraction");
                while (i < s.size() && s[i] >= '0' && s[i] <= '9') ++i;
            }
            if (i < s.size() && (s[i] == 'e' || s[i] == 'E')) {
                ++i;
                if (i < s.size() && (s[i] == '+' || s[i] == '-')) ++i;
                if (i >= s.size() || !(s[i] >= '0' && s[i] <= '9')) fail("bad exponent");
                while (i < s.size() && s[i] >= '0' && s[i] <= '9') ++i;
            }
            return std::strtod(s.substr(start, i - start).c_str(), nullptr);
        }
        static void utf8(std::string& o, std::uint32_t cp) {
            if (cp < 0x80) {
                o += static_cast<char>(cp);
            } else if (cp < 0x800) {
                o += static_cast<char>(0xC0 | (cp >> 6));
                o += static_cast<char>(0x80 | (cp & 0x3F));
            } else if (cp < 0x10000) {
                o += static_cast<char>(0xE0 | (cp >> 12));
                o += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
                o += static_cast<char>(0x80 | (cp & 0x3F));
            } else {
                o += static_cast<char>(0xF0 | (cp >> 18));
                o += static_cast<char>(0x80 | ((cp >> 12) & 0x3F));
                o += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
                o += static_cast<char>(0x80 | (cp & 0x3F));
            }
        }
        std::uint32_t hex4() {
            if (i + 4 > s.size()) fail("bad \\u escape");
            std::uint32_t v = 0;
            for (int k = 0; k < 4; ++k) {
                const char h = s[i++];
                v <<= 4;
                if (h >= '0' && h <= '9') v |= h - '0';
                else if (h >= 'a' && h <= 'f') v |= h - 'a' + 10;
                else if (h >= 'A' && h <= 'F') v |= h - 'A' + 10;
                else fail("bad hex digit");
            }
            return v;
        }
        std::string string() {
            ++i;  // opening quote
            std::string o;
            while (true) {
                if (i >= s.size()) fail("unterminated string");
                const char c = s[i++];
                if (c == '"') break;
                if (static_cast<unsigned char>(c) < 0x20) fail("control character in string");
                if (c != '\\') { o += c; continue; }
                if (i >= s.size()) fail("bad escape");
                const char e = s[i++];
                switch (e) {
                    case '"': o += '"'; break;
                    case '\\': o += '\\'; break;
                    case '/': o += '/'; break;
                    case 'b': o += '\b'; break;
                    case 'f': o += '\f'; break;
                    case 'n': o += '\n'; break;
                    case 'r': o += '\r'; break;
                    case 't': o += '\t'; break;
                    case 'u': {
                        std::uint32_t cp = hex4();
                        if (cp >= 0xD800 && cp <= 0xDBFF) {
                            if (i + 2 <= s.size() && s[i] == '\\' && s[i + 1] == 'u') {
                                i += 2;
                                const std::uint32_t lo = hex4();
                                if (lo < 0xDC00 || lo > 0xDFFF) fail("bad surrogate pair");
                                cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                            } else {
                                fail("lone surrogate");
                            }
                        }
                        utf8(o, cp);
                        break;
                    }
                    default: fail("bad escape");
                }
            }
            return o;
        }
    };
};

}  // namespace water::scene
