// hydrant_gb300_json.hpp -- a small JSON value, reader and writer (C++17).
//
// Used for the dataset description (package_meta.json) and for the renderer
// configuration objects the C++ layer accepts (RendererConfig, CameraConfig,
// the per-renderer params; renderer.schema.hpp, scene.schema.hpp and the
// *.schema.hpp files of the reference).  Numbers are doubles; objects keep
// their keys sorted (std::map); parse errors throw hygb::json::ParseError
// with the byte offset.
#pragma once

#include <cmath>
#include <cstdint>
#include <cstdio>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace hygb {
namespace json {

struct ParseError : std::runtime_error {
    size_t offset;
    ParseError(const std::string &what, size_t at)
        : std::runtime_error("json: " + what + " at byte " + std::to_string(at)), offset(at) {}
};

class Value {
public:
    enum Kind { Null, Bool, Number, String, Array, Object };
    using array_t = std::vector<Value>;
    using object_t = std::map<std::string, Value>;

    Value() = default;
    Value(std::nullptr_t) {}
    Value(bool b) : kind_(Bool), b_(b) {}
    Value(double d) : kind_(Number), d_(d) {}
    Value(int i) : kind_(Number), d_(double(i)) {}
    Value(long long i) : kind_(Number), d_(double(i)) {}
    Value(const char *s) : kind_(String), s_(s) {}
    Value(std::string s) : kind_(String), s_(std::move(s)) {}
    Value(array_t a) : kind_(Array), a_(std::make_shared<array_t>(std::move(a))) {}
    Value(object_t o) : kind_(Object), o_(std::make_shared<object_t>(std::move(o))) {}

    Kind kind() const { return kind_; }
    bool is_null() const { return kind_ == Null; }
    bool is_number() const { return kind_ == Number; }
    bool is_string() const { return kind_ == String; }
    bool is_array() const { return kind_ == Array; }
    bool is_object() const { return kind_ == Object; }

    bool as_bool() const { return need(Bool, "a boolean"), b_; }
    double as_number() const { return need(Number, "a number"), d_; }
    long long as_int() const {
        need(Number, "a number");
        if (d_ != std::floor(d_)) throw std::runtime_error("json: expected an integer");
        return (long long)d_;
    }
    const std::string &as_string() const { return need(String, "a string"), s_; }
    const array_t &as_array() const { return need(Array, "an array"), *a_; }
    const object_t &as_object() const { return need(Object, "an object"), *o_; }
    array_t &as_array() { return need(Array, "an array"), *a_; }
    object_t &as_object() { return need(Object, "an object"), *o_; }

    size_t size() const {
        if (kind_ == Array) return a_->size();
        if (kind_ == Object) return o_->size();
        return 0;
    }
    const Value &operator[](size_t i) const { return as_array().at(i); }
    const Value &operator[](int i) const { return as_array().at(size_t(i)); }
    bool has(const std::string &k) const { return kind_ == Object && o_->count(k) != 0; }
    // member lookup; a missing key reads as null
    const Value &operator[](const std::string &k) const {
        static const Value null_value;
        if (kind_ != Object) return null_value;
        auto it = o_->find(k);
        return it == o_->end() ? null_value : it->second;
    }
    const Value &operator[](const char *k) const { return (*this)[std::string(k)]; }
    Value &set(const std::string &k, Value v) {
        if (kind_ == Null) *this = Value(object_t{});
        as_object()[k] = std::move(v);
        return *this;
    }
    Value &push(Value v) {
        if (kind_ == Null) *this = Value(array_t{});
        as_array().push_back(std::move(v));
        return *this;
    }

    // convenience readers with defaults for absent members
    double number_or(const std::string &k, double dflt) const {
        const Value &v = (*this)[k];
        return v.is_null() ? dflt : v.as_number();
    }
    std::string string_or(const std::string &k, const std::string &dflt) const {
        const Value &v = (*this)[k];
        return v.is_null() ? dflt : v.as_string();
    }

    std::string dump(int indent = -1) const {
        std::string out;
        write(out, indent, 0);
        return out;
    }

private:
    Kind kind_ = Null;
    bool b_ = false;
    double d_ = 0.0;
    std::string s_;
    std::shared_ptr<array_t> a_;
    std::shared_ptr<object_t> o_;

    void need(Kind k, const char *what) const {
        if (kind_ != k) throw std::runtime_error(std::string("json: expected ") + what);
    }

    static void write_string(std::string &out, const std::string &s) {
        out += '"';
        for (unsigned char c : s) {
            switch (c) {
                case '"': out += "\\\""; break;
                case '\\': out += "\\\\"; break;
                case '\n': out += "\\n"; break;
                case '\r': out += "\\r"; break;
                case '\t': out += "\\t"; break;
                case '\b': out += "\\b"; break;
                case '\f': out += "\\f"; break;
                default:
                    if (c < 0x20) {
                        char buf[8];
                        std::snprintf(buf, sizeof(buf), "\\u%04x", c);
                        out += buf;
                    } else {
                        out += char(c);
                    }
            }
        }
        out += '"';
    }

    void write(std::string &out, int indent, int depth) const {
        auto nl = [&](int d) {
            if (indent < 0) return;
            out += '\n';
            out.append(size_t(indent) * d, ' ');
        };
        switch (kind_) {
            case Null: out += "null"; break;
            case Bool: out += b_ ? "true" : "false"; break;
            case Number: {
                if (std::isfinite(d_) && d_ == std::floor(d_) && std::fabs(d_) < 9.0e15) {
                    out += std::to_string((long long)d_);
                } else {
                    char buf[32];
                    std::snprintf(buf, sizeof(buf), "%.17g", d_);
                    out += buf;
                }
                break;
            }
            case String: write_string(out, s_); break;
            case Array: {
                out += '[';
                for (size_t i = 0; i < a_->size(); ++i) {
                    if (i) out += ',';
                    nl(depth + 1);
                    (*a_)[i].write(out, indent, depth + 1);
                }
                if (!a_->empty()) nl(depth);
                out += ']';
                break;
            }
            case Object: {
                out += '{';
                bool first = true;
                for (auto &kv : *o_) {
                    if (!first) out += ',';
                    first = false;
                    nl(depth + 1);
                    write_string(out, kv.first);
                    out += indent < 0 ? ":" : ": ";
                    kv.second.write(out, indent, depth + 1);
                }
                if (!o_->empty()) nl(depth);
                out += '}';
                break;
            }
        }
    }
};

namespace detail {

class Reader {
public:
    explicit Reader(const std::string &text) : t_(text) {}

    Value document() {
        Value v = value(0);
        ws();
        if (i_ != t_.size()) fail("trailing characters");
        return v;
    }

private:
    const std::string &t_;
    size_t i_ = 0;

    [[noreturn]] void fail(const std::string &what) const { throw ParseError(what, i_); }

    void ws() {
        while (i_ < t_.size() && (t_[i_] == ' ' || t_[i_] == '\t' || t_[i_] == '\n' || t_[i_] == '\r'))
            ++i_;
    }

    bool literal(const char *word) {
        size_t n = 0;
        while (word[n]) ++n;
        if (t_.compare(i_, n, word) != 0) return false;
        i_ += n;
        return true;
    }

    Value value(int depth) {
        if (depth > 256) fail("nesting too deep");
        ws();
        if (i_ >= t_.size()) fail("unexpected end");
        const char c = t_[i_];
        if (c == '{') return object(depth);
        if (c == '[') return array(depth);
        if (c == '"') return Value(string());
        if (c == 't') {
            if (!literal("true")) fail("bad literal");
            return Value(true);
        }
        if (c == 'f') {
            if (!literal("false")) fail("bad literal");
            return Value(false);
        }
        if (c == 'n') {
            if (!literal("null")) fail("bad literal");
            return Value();
        }
        if (c == '-' || (c >= '0' && c <= '9')) return Value(number());
        fail(std::string("unexpected character '") + c + "'");
    }

    Value object(int depth) {
        ++i_;  // {
        Value::object_t o;
        ws();
        if (i_ < t_.size() && t_[i_] == '}') {
            ++i_;
            return Value(std::move(o));
        }
        for (;;) {
            ws();
            if (i_ >= t_.size() || t_[i_] != '"') fail("expected a key");
            std::string k = string();
            ws();
            if (i_ >= t_.size() || t_[i_] != ':') fail("expected ':'");
            ++i_;
            o[k] = value(depth + 1);
            ws();
            if (i_ >= t_.size()) fail("unexpected end in object");
            if (t_[i_] == ',') {
                ++i_;
                continue;
            }
            if (t_[i_] == '}') {
                ++i_;
                return Value(std::move(o));
            }
            fail("expected ',' or '}'");
        }
    }

    Value array(int depth) {
        ++i_;  // [
        Value::array_t a;
        ws();
        if (i_ < t_.size() && t_[i_] == ']') {
            ++i_;
            return Value(std::move(a));
        }
        for (;;) {
            a.push_back(value(depth + 1));
            ws();
            if (i_ >= t_.size()) fail("unexpected end in array");
            if (t_[i_] == ',') {
                ++i_;
                continue;
            }
            if (t_[i_] == ']') {
                ++i_;
                return Value(std::move(a));
            }
            fail("expected ',' or ']'");
        }
    }

    static void utf8(std::string &out, uint32_t cp) {
        if (cp < 0x80) {
            out += char(cp);
        } else if (cp < 0x800) {
            out += char(0xC0 | (cp >> 6));
            out += char(0x80 | (cp & 0x3F));
        } else if (cp < 0x10000) {
            out += char(0xE0 | (cp >> 12));
            out += char(0x80 | ((cp >> 6) & 0x3F));
            out += char(0x80 | (cp & 0x3F));
        } else {
            out += char(0xF0 | (cp >> 18));
            out += char(0x80 | ((cp >> 12) & 0x3F));
            out += char(0x80 | ((cp >> 6) & 0x3F));
            out += char(0x80 | (cp & 0x3F));
        }
    }

    uint32_t hex4() {
        if (i_ + 4 > t_.size()) fail("short \\u escape");
        uint32_t v = 0;
        for (int k = 0; k < 4; ++k) {
            const char h = t_[i_++];
            v <<= 4;
            if (h >= '0' && h <= '9') v |= uint32_t(h - '0');
            else if (h >= 'a' && h <= 'f') v |= uint32_t(h - 'a' + 10);
            else if (h >= 'A' && h <= 'F') v |= uint32_t(h - 'A' + 10);
            else fail("bad hex digit");
        }
        return v;
    }

    std::string string() {
        ++i_;  // opening quote
        std::string out;
        for (;;) {
            if (i_ >= t_.size()) fail("unterminated string");
            const char c = t_[i_++];
            if (c == '"') return out;
            if (static_cast<unsigned char>(c) < 0x20) fail("control character in string");
            if (c != '\\') {
                out += c;
                continue;
            }
            if (i_ >= t_.size()) fail("unterminated escape");
            const char e = t_[i_++];
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
                    uint32_t cp = hex4();
                    if (cp >= 0xD800 && cp < 0xDC00) {  // surrogate pair
                        if (i_ + 2 > t_.size() || t_[i_] != '\\' || t_[i_ + 1] != 'u')
                            fail("lone surrogate");
                        i_ += 2;
                        const uint32_t lo = hex4();
                        if (lo < 0xDC00 || lo >= 0xE000) fail("bad surrogate pair");
                        cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                    }
                    utf8(out, cp);
                    break;
                }
                default: fail("bad escape");
            }
        }
    }

    double number() {
        const size_t start = i_;
        if (t_[i_] == '-') ++i_;
        if (i_ >= t_.size()) fail("bad number");
        if (t_[i_] == '0') {
            ++i_;
        } else if (t_[i_] >= '1' && t_[i_] <= '9') {
            while (i_ < t_.size() && t_[i_] >= '0' && t_[i_] <= '9') ++i_;
        } else {
            fail("bad number");
        }
        if (i_ < t_.size() && t_[i_] == '.') {
            ++i_;
            if (i_ >= t_.size() || t_[i_] < '0' || t_[i_] > '9') fail("bad fraction");
            while (i_ < t_.size() && t_[i_] >= '0' && t_[i_] <= '9') ++i_;
        }
        if (i_ < t_.size() && (t_[i_] == 'e' || t_[i_] == 'E')) {
            ++i_;
            if (i_ < t_.size() && (t_[i_] == '+' || t_[i_] == '-')) ++i_;
            if (i_ >= t_.size() || t_[i_] < '0' || t_[i_] > '9') fail("bad exponent");
            while (i_ < t_.size() && t_[i_] >= '0' && t_[i_] <= '9') ++i_;
        }
        // strtod on a copy: the text is locale-independent JSON
        return std::strtod(t_.substr(start, i_ - start).c_str(), nullptr);
    }
};

}  // namespace detail

inline Value parse(const std::string &text) { return detail::Reader(text).document(); }

}  // namespace json
}  // namespace hygb
