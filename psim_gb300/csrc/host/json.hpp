// Minimal JSON document reader for psim model files.
//
// psim model files are written by psim_python's ModelBuilder.export
// (psim_python/psim/builder_tools.py:546-576) and read by the reference with
// nlohmann::json (psim/src/inputManager.cpp:14-115).  nlohmann is not a
// dependency of this project, so this header provides the small subset the
// model loader needs: objects, arrays, numbers, strings, booleans and null.
// Numbers keep both their double value and, when written without a fraction
// or exponent, their exact 64-bit integer value.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <fstream>
#include <map>
#include <memory>
#include <sstream>
#include <stdexcept>
#include <string>
#include <vector>

namespace psim_json {

class Value {
public:
    enum class Kind { Null, Bool, Number, String, Array, Object };

    Value() = default;

    Kind kind() const noexcept { return kind_; }
    bool is_object() const noexcept { return kind_ == Kind::Object; }
    bool is_array() const noexcept { return kind_ == Kind::Array; }
    bool is_number() const noexcept { return kind_ == Kind::Number; }

    // Object member access; throws std::out_of_range like nlohmann::json::at.
    const Value& at(const std::string& key) const {
        if (kind_ != Kind::Object) { throw std::runtime_error("JSON value is not an object (key '" + key + "')"); }
        const auto it = object_.find(key);
        if (it == object_.end()) { throw std::out_of_range("JSON key not found: '" + key + "'"); }
        return it->second;
    }
    bool contains(const std::string& key) const { return kind_ == Kind::Object && object_.count(key) != 0; }

    const Value& at(std::size_t index) const {
        if (kind_ != Kind::Array) { throw std::runtime_error("JSON value is not an array"); }
        return array_.at(index);
    }
    std::size_t size() const noexcept {
        return kind_ == Kind::Array ? array_.size() : (kind_ == Kind::Object ? object_.size() : 0);
    }
    const std::vector<Value>& items() const {
        if (kind_ != Kind::Array) { throw std::runtime_error("JSON value is not an array"); }
        return array_;
    }

    double as_double() const {
        if (kind_ == Kind::Number) { return number_; }
        if (kind_ == Kind::Bool) { return bool_ ? 1.0 : 0.0; }
        throw std::runtime_error("JSON value is not a number");
    }
    // Integer conversion: exact for integer literals, truncation of the double otherwise.
    std::int64_t as_int() const {
        if (kind_ == Kind::Number) { return is_integer_ ? integer_ : static_cast<std::int64_t>(number_); }
        if (kind_ == Kind::Bool) { return bool_ ? 1 : 0; }
        throw std::runtime_error("JSON value is not a number");
    }
    bool as_bool() const {
        if (kind_ == Kind::Bool) { return bool_; }
        throw std::runtime_error("JSON value is not a boolean");
    }
    const std::string& as_string() const {
        if (kind_ != Kind::String) { throw std::runtime_error("JSON value is not a string"); }
        return string_;
    }

private:
    friend class Parser;
    Kind kind_{ Kind::Null };
    bool bool_{ false };
    double number_{ 0.0 };
    bool is_integer_{ false };
    std::int64_t integer_{ 0 };
    std::string string_;
    std::vector<Value> array_;
    std::map<std::string, Value> object_;
};

class Parser {
public:
    explicit Parser(const std::string& text) : s_{ text } {}

    Value parse_document() {
        Value v = parse_value();
        skip_ws();
        if (pos_ != s_.size()) { fail("trailing characters after JSON document"); }
        return v;
    }

private:
    const std::string& s_;
    std::size_t pos_{ 0 };

    [[noreturn]] void fail(const std::string& what) const {
        throw std::runtime_error("JSON parse error at offset " + std::to_string(pos_) + ": " + what);
    }
    void skip_ws() {
        while (pos_ < s_.size() && (s_[pos_] == ' ' || s_[pos_] == '\n' || s_[pos_] == '\r' || s_[pos_] == '\t')) {
            ++pos_;
        }
    }
    char peek() {
        skip_ws();
        if (pos_ >= s_.size()) { fail("unexpected end of input"); }
        return s_[pos_];
    }
    void expect(char c) {
        if (peek() != c) { fail(std::string("expected '") + c + "'"); }
        ++pos_;
    }
    bool match_word(const char* w) {
        std::size_t n = 0;
        while (w[n] != '\0') { ++n; }
        if (s_.compare(pos_, n, w) == 0) {
            pos_ += n;
            return true;
        }
        return false;
    }

    Value parse_value() {
        const char c = peek();
        Value v;
        if (c == '{') {
            v.kind_ = Value::Kind::Object;
            ++pos_;
            if (peek() == '}') {
                ++pos_;
                return v;
            }
            while (true) {
                if (peek() != '"') { fail("expected object key"); }
                std::string key = parse_string();
                expect(':');
                v.object_[key] = parse_value();
                const char d = peek();
                ++pos_;
                if (d == '}') { break; }
                if (d != ',') { fail("expected ',' or '}' in object"); }
            }
        } else if (c == '[') {
            v.kind_ = Value::Kind::Array;
            ++pos_;
            if (peek() == ']') {
                ++pos_;
                return v;
            }
            while (true) {
                v.array_.push_back(parse_value());
                const char d = peek();
                ++pos_;
                if (d == ']') { break; }
                if (d != ',') { fail("expected ',' or ']' in array"); }
            }
        } else if (c == '"') {
            v.kind_ = Value::Kind::String;
            v.string_ = parse_string();
        } else if (match_word("true")) {
            v.kind_ = Value::Kind::Bool;
            v.bool_ = true;
        } else if (match_word("false")) {
            v.kind_ = Value::Kind::Bool;
            v.bool_ = false;
        } else if (match_word("null")) {
            v.kind_ = Value::Kind::Null;
        } else {
            parse_number(v);
        }
        return v;
    }

    std::string parse_string() {
        expect('"');
        std::string out;
        while (true) {
            if (pos_ >= s_.size()) { fail("unterminated string"); }
            const char c = s_[pos_++];
            if (c == '"') { break; }
            if (c == '\\') {
                if (pos_ >= s_.size()) { fail("bad escape"); }
                const char e = s_[pos_++];
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
                    if (pos_ + 4 > s_.size()) { fail("bad \\u escape"); }
                    const unsigned cp = static_cast<unsigned>(std::strtoul(s_.substr(pos_, 4).c_str(), nullptr, 16));
                    pos_ += 4;
                    // Model files only carry ASCII names; encode the BMP code point as UTF-8.
                    if (cp < 0x80U) {
                        out.push_back(static_cast<char>(cp));
                    } else if (cp < 0x800U) {
                        out.push_back(static_cast<char>(0xC0U | (cp >> 6U)));
                        out.push_back(static_cast<char>(0x80U | (cp & 0x3FU)));
                    } else {
                        out.push_back(static_cast<char>(0xE0U | (cp >> 12U)));
                        out.push_back(static_cast<char>(0x80U | ((cp >> 6U) & 0x3FU)));
                        out.push_back(static_cast<char>(0x80U | (cp & 0x3FU)));
                    }
                    break;
                }
                default: fail("bad escape");
                }
            } else {
                out.push_back(c);
            }
        }
        return out;
    }

    void parse_number(Value& v) {
        const std::size_t start = pos_;
        bool integral = true;
        if (pos_ < s_.size() && (s_[pos_] == '-' || s_[pos_] == '+')) { ++pos_; }
        while (pos_ < s_.size()) {
            const char c = s_[pos_];
            if (c >= '0' && c <= '9') {
                ++pos_;
            } else if (c == '.' || c == 'e' || c == 'E' || c == '-' || c == '+') {
                integral = false;
                ++pos_;
            } else {
                break;
            }
        }
        if (pos_ == start) { fail("unexpected character"); }
        const std::string tok = s_.substr(start, pos_ - start);
        char* end = nullptr;
        v.kind_ = Value::Kind::Number;
        v.number_ = std::strtod(tok.c_str(), &end);
        if (end == nullptr || *end != '\0') { fail("malformed number '" + tok + "'"); }
        if (integral) {
            v.is_integer_ = true;
            v.integer_ = std::strtoll(tok.c_str(), nullptr, 10);
        }
    }
};

inline Value parse(const std::string& text) {
    Parser p{ text };
    return p.parse_document();
}

inline Value parse_file(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f.is_open()) { throw std::runtime_error("Error opening file at " + path); }
    std::ostringstream ss;
    ss << f.rdbuf();
    return parse(ss.str());
}

}// namespace psim_json
