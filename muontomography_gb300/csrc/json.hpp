// Minimal JSON value + parser for the reconstruction configs.
//
// The reference reads its configs with nlohmann::json (include/MutoConfig.h:7-46)
// through `config.at(key)`, `config.value(key, default)`, `config[key]` and
// `config.find(key)`.  This header gives the same operations on a small value
// type of its own: objects keep insertion order, numbers remember whether they
// were written as integers, and `value()` converts to the type of the default
// (an integer default accepts any number and truncates it, a bool default
// needs true/false, a string default needs a string) and throws
// muto::json::type_error on a mismatch, like nlohmann does.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <type_traits>
#include <utility>
#include <vector>

namespace muto {

class json {
public:
    enum class kind { null, boolean, number, string, array, object };

    struct parse_error : std::runtime_error {
        using std::runtime_error::runtime_error;
    };
    struct type_error : std::runtime_error {
        using std::runtime_error::runtime_error;
    };
    struct out_of_range : std::runtime_error {
        using std::runtime_error::runtime_error;
    };

    json() = default;
    json(bool b) : k_(kind::boolean), b_(b) {}
    json(double d) : k_(kind::number), d_(d) {}
    json(int i) : k_(kind::number), d_(i), integral_(true) {}
    json(int64_t i) : k_(kind::number), d_(static_cast<double>(i)), integral_(true) {}
    json(const char* s) : k_(kind::string), s_(s) {}
    json(std::string s) : k_(kind::string), s_(std::move(s)) {}

    static json parse(const std::string& text) {
        size_t pos = 0;
        json v = parse_value(text, pos, 0);
        skip_ws(text, pos);
        if (pos != text.size()) throw parse_error("trailing characters at offset " + std::to_string(pos));
        return v;
    }

    kind type() const { return k_; }
    bool is_object() const { return k_ == kind::object; }
    bool is_array() const { return k_ == kind::array; }
    bool is_number() const { return k_ == kind::number; }
    bool is_string() const { return k_ == kind::string; }
    bool is_boolean() const { return k_ == kind::boolean; }
    bool is_null() const { return k_ == kind::null; }
    bool is_integral() const { return k_ == kind::number && integral_; }

    size_t size() const {
        if (k_ == kind::array) return arr_.size();
        if (k_ == kind::object) return obj_.size();
        return k_ == kind::null ? 0 : 1;
    }

    bool contains(const std::string& key) const { return find_key(key) != nullptr; }

    const json& at(const std::string& key) const {
        const json* v = find_key(key);
        if (!v) throw out_of_range("key '" + key + "' not found");
        return *v;
    }
    const json& at(size_t i) const {
        if (k_ != kind::array || i >= arr_.size()) throw out_of_range("array index out of range");
        return arr_[i];
    }
    // nlohmann's non-const operator[] inserts null for a missing key; the
    // const form here returns a shared null instead.
    const json& operator[](const std::string& key) const {
        const json* v = find_key(key);
        return v ? *v : null_value();
    }
    const json& operator[](size_t i) const { return at(i); }

    double get_double() const {
        if (k_ != kind::number) throw type_error("type must be number");
        return d_;
    }
    int64_t get_int() const {
        if (k_ != kind::number) throw type_error("type must be number");
        return static_cast<int64_t>(d_);
    }
    bool get_bool() const {
        if (k_ != kind::boolean) throw type_error("type must be boolean");
        return b_;
    }
    const std::string& get_string() const {
        if (k_ != kind::string) throw type_error("type must be string");
        return s_;
    }
    const std::vector<json>& items() const {
        if (k_ != kind::array) throw type_error("type must be array");
        return arr_;
    }
    const std::vector<std::pair<std::string, json>>& members() const {
        if (k_ != kind::object) throw type_error("type must be object");
        return obj_;
    }

    // value(key, default) with the default's type (nlohmann basic_json::value)
    double value(const std::string& key, double def) const {
        const json* v = object_key(key);
        return v ? v->get_double() : def;
    }
    int value(const std::string& key, int def) const {
        const json* v = object_key(key);
        return v ? static_cast<int>(v->get_int()) : def;
    }
    int64_t value(const std::string& key, int64_t def) const {
        const json* v = object_key(key);
        return v ? v->get_int() : def;
    }
    bool value(const std::string& key, bool def) const {
        const json* v = object_key(key);
        return v ? v->get_bool() : def;
    }
    std::string value(const std::string& key, const char* def) const {
        const json* v = object_key(key);
        return v ? v->get_string() : std::string(def);
    }
    std::string value(const std::string& key, const std::string& def) const {
        const json* v = object_key(key);
        return v ? v->get_string() : def;
    }

    std::string dump() const {
        std::string out;
        dump_to(out);
        return out;
    }

    // Implicit conversions (nlohmann's `operator ValueType()`): a number to
    // any arithmetic type (truncated towards zero for integers), a boolean to
    // bool, a string to std::string, an array to std::vector of any of these;
    // a value of another kind throws type_error.  They let code written for
    // nlohmann::json, such as `int n = config.get("detector_middle");` in the
    // reference's driver, compile against this type unchanged.
    template <typename T, typename std::enable_if<std::is_arithmetic<T>::value, int>::type = 0>
    operator T() const {
        if (std::is_same<T, bool>::value) return static_cast<T>(get_bool());
        return static_cast<T>(get_double());
    }
    operator std::string() const { return get_string(); }
    template <typename T>
    operator std::vector<T>() const {
        std::vector<T> out;
        for (const json& e : items()) out.push_back(static_cast<T>(e));
        return out;
    }

private:
    kind k_ = kind::null;
    bool b_ = false;
    double d_ = 0.0;
    bool integral_ = false;
    std::string s_;
    std::vector<json> arr_;
    std::vector<std::pair<std::string, json>> obj_;

    static const json& null_value() {
        static const json n;
        return n;
    }

    const json* find_key(const std::string& key) const {
        if (k_ != kind::object) return nullptr;
        for (const auto& kv : obj_)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    const json* object_key(const std::string& key) const {
        if (k_ != kind::object) throw type_error("cannot use value() with a non-object");
        return find_key(key);
    }

    static void skip_ws(const std::string& t, size_t& p) {
        while (p < t.size() && (t[p] == ' ' || t[p] == '\n' || t[p] == '\r' || t[p] == '\t')) ++p;
    }

    static json parse_value(const std::string& t, size_t& p, int depth) {
        if (depth > 64) throw parse_error("nesting too deep");
        skip_ws(t, p);
        if (p >= t.size()) throw parse_error("unexpected end of input");
        const char c = t[p];
        if (c == '{') return parse_object(t, p, depth);
        if (c == '[') return parse_array(t, p, depth);
        if (c == '"') return json(parse_string(t, p));
        if (t.compare(p, 4, "true") == 0) { p += 4; return json(true); }
        if (t.compare(p, 5, "false") == 0) { p += 5; return json(false); }
        if (t.compare(p, 4, "null") == 0) { p += 4; return json(); }
        return parse_number(t, p);
    }

    static json parse_number(const std::string& t, size_t& p) {
        const size_t b = p;
        if (p < t.size() && t[p] == '-') ++p;
        bool integral = true;
        auto digits = [&]() {
            const size_t s = p;
            while (p < t.size() && t[p] >= '0' && t[p] <= '9') ++p;
            return p > s;
        };
        if (!digits()) throw parse_error("invalid number at offset " + std::to_string(b));
        if (p < t.size() && t[p] == '.') {
            ++p;
            integral = false;
            if (!digits()) throw parse_error("invalid number at offset " + std::to_string(b));
        }
        if (p < t.size() && (t[p] == 'e' || t[p] == 'E')) {
            ++p;
            integral = false;
            if (p < t.size() && (t[p] == '+' || t[p] == '-')) ++p;
            if (!digits()) throw parse_error("invalid number at offset " + std::to_string(b));
        }
        json v(std::strtod(t.c_str() + b, nullptr));
        v.integral_ = integral;
        return v;
    }

    static void put_utf8(std::string& out, uint32_t cp) {
        if (cp < 0x80) out += static_cast<char>(cp);
        else if (cp < 0x800) {
            out += static_cast<char>(0xC0 | (cp >> 6));
            out += static_cast<char>(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += static_cast<char>(0xE0 | (cp >> 12));
            out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
            out += static_cast<char>(0x80 | (cp & 0x3F));
        } else {
            out += static_cast<char>(0xF0 | (cp >> 18));
            out += static_cast<char>(0x80 | ((cp >> 12) & 0x3F));
            out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
            out += static_cast<char>(0x80 | (cp & 0x3F));
        }
    }

    static uint32_t hex4(const std::string& t, size_t p) {
        if (p + 4 > t.size()) throw parse_error("bad \\u escape");
        uint32_t v = 0;
        for (size_t i = p; i < p + 4; ++i) {
            const char c = t[i];
            v <<= 4;
            if (c >= '0' && c <= '9') v |= static_cast<uint32_t>(c - '0');
            else if (c >= 'a' && c <= 'f') v |= static_cast<uint32_t>(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F') v |= static_cast<uint32_t>(c - 'A' + 10);
            else throw parse_error("bad \\u escape");
        }
        return v;
    }

    static std::string parse_string(const std::string& t, size_t& p) {
        ++p;  // opening quote
        std::string out;
        while (true) {
            if (p >= t.size()) throw parse_error("unterminated string");
            const char c = t[p++];
            if (c == '"') break;
            if (c != '\\') { out += c; continue; }
            if (p >= t.size()) throw parse_error("unterminated escape");
            const char e = t[p++];
            switch (e) {
                case '"': out += '"'; break;
                case '\\': out += '\\'; break;
                case '/': out += '/'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'n': out += '\n'; break;
                case 'r': out += '\r'; break;
                case 't': out += '\t'; break;
                case 'u': {
                    uint32_t cp = hex4(t, p);
                    p += 4;
                    if (cp >= 0xD800 && cp < 0xDC00 && p + 6 <= t.size() && t[p] == '\\' && t[p + 1] == 'u') {
                        const uint32_t lo = hex4(t, p + 2);
                        if (lo >= 0xDC00 && lo < 0xE000) {
                            cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                            p += 6;
                        }
                    }
                    put_utf8(out, cp);
                    break;
                }
                default: throw parse_error("bad escape");
            }
        }
        return out;
    }

    static json parse_array(const std::string& t, size_t& p, int depth) {
        json v;
        v.k_ = kind::array;
        ++p;
        skip_ws(t, p);
        if (p < t.size() && t[p] == ']') { ++p; return v; }
        while (true) {
            v.arr_.push_back(parse_value(t, p, depth + 1));
            skip_ws(t, p);
            if (p >= t.size()) throw parse_error("unterminated array");
            if (t[p] == ',') { ++p; continue; }
            if (t[p] == ']') { ++p; return v; }
            throw parse_error("expected ',' or ']' at offset " + std::to_string(p));
        }
    }

    static json parse_object(const std::string& t, size_t& p, int depth) {
        json v;
        v.k_ = kind::object;
        ++p;
        skip_ws(t, p);
        if (p < t.size() && t[p] == '}') { ++p; return v; }
        while (true) {
            skip_ws(t, p);
            if (p >= t.size() || t[p] != '"') throw parse_error("expected key at offset " + std::to_string(p));
            std::string key = parse_string(t, p);
            skip_ws(t, p);
            if (p >= t.size() || t[p] != ':') throw parse_error("expected ':' at offset " + std::to_string(p));
            ++p;
            json val = parse_value(t, p, depth + 1);
            bool replaced = false;  // a repeated key keeps the last value, like nlohmann
            for (auto& kv : v.obj_)
                if (kv.first == key) { kv.second = val; replaced = true; }
            if (!replaced) v.obj_.emplace_back(std::move(key), std::move(val));
            skip_ws(t, p);
            if (p >= t.size()) throw parse_error("unterminated object");
            if (t[p] == ',') { ++p; continue; }
            if (t[p] == '}') { ++p; return v; }
            throw parse_error("expected ',' or '}' at offset " + std::to_string(p));
        }
    }

    static void dump_string(std::string& out, const std::string& s) {
        out += '"';
        for (const char c : s) {
            switch (c) {
                case '"': out += "\\\""; break;
                case '\\': out += "\\\\"; break;
                case '\n': out += "\\n"; break;
                case '\r': out += "\\r"; break;
                case '\t': out += "\\t"; break;
                default:
                    if (static_cast<unsigned char>(c) < 0x20) {
                        char buf[8];
                        std::snprintf(buf, sizeof buf, "\\u%04x", static_cast<unsigned>(c));
                        out += buf;
                    } else {
                        out += c;
                    }
            }
        }
        out += '"';
    }

    void dump_to(std::string& out) const {
        switch (k_) {
            case kind::null: out += "null"; break;
            case kind::boolean: out += b_ ? "true" : "false"; break;
            case kind::number: {
                char buf[40];
                if (integral_ && std::fabs(d_) < 9.0e15) std::snprintf(buf, sizeof buf, "%lld", static_cast<long long>(d_));
                else std::snprintf(buf, sizeof buf, "%.17g", d_);
                out += buf;
                break;
            }
            case kind::string: dump_string(out, s_); break;
            case kind::array:
                out += '[';
                for (size_t i = 0; i < arr_.size(); ++i) {
                    if (i) out += ',';
                    arr_[i].dump_to(out);
                }
                out += ']';
                break;
            case kind::object:
                out += '{';
                for (size_t i = 0; i < obj_.size(); ++i) {
                    if (i) out += ',';
                    dump_string(out, obj_[i].first);
                    out += ':';
                    obj_[i].second.dump_to(out);
                }
                out += '}';
                break;
        }
    }
};

}  // namespace muto
