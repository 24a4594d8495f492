// Minimal JSON value + parser + writer for the tiny-cuda-nn style configuration objects
// ("encoding", "network", "loss", "optimizer") and the Trainer checkpoint format.
// Numbers are held as double; object key order is preserved.
#pragma once

#include <cstdint>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace nlod {

class Json {
public:
    enum class Type { Null, Bool, Number, String, Array, Object };

    Json() = default;
    static Json number(double v) { Json j; j.t_ = Type::Number; j.num_ = v; return j; }
    static Json boolean(bool v) { Json j; j.t_ = Type::Bool; j.b_ = v; return j; }
    static Json string(std::string s) { Json j; j.t_ = Type::String; j.str_ = std::move(s); return j; }
    static Json array() { Json j; j.t_ = Type::Array; return j; }
    static Json object() { Json j; j.t_ = Type::Object; return j; }

    Type type() const { return t_; }
    bool is_null() const { return t_ == Type::Null; }
    bool is_number() const { return t_ == Type::Number; }
    bool is_bool() const { return t_ == Type::Bool; }
    bool is_string() const { return t_ == Type::String; }
    bool is_array() const { return t_ == Type::Array; }
    bool is_object() const { return t_ == Type::Object; }

    double as_number() const {
        if (t_ == Type::Number) return num_;
        if (t_ == Type::Bool) return b_ ? 1.0 : 0.0;
        throw std::runtime_error("json: value is not a number");
    }
    bool as_bool() const {
        if (t_ == Type::Bool) return b_;
        if (t_ == Type::Number) return num_ != 0.0;
        throw std::runtime_error("json: value is not a boolean");
    }
    const std::string& as_string() const {
        if (t_ != Type::String) throw std::runtime_error("json: value is not a string");
        return str_;
    }
    const std::vector<Json>& items() const {
        if (t_ != Type::Array) throw std::runtime_error("json: value is not an array");
        return arr_;
    }
    std::vector<Json>& items() {
        if (t_ != Type::Array) throw std::runtime_error("json: value is not an array");
        return arr_;
    }
    const std::vector<std::pair<std::string, Json>>& members() const {
        if (t_ != Type::Object) throw std::runtime_error("json: value is not an object");
        return obj_;
    }

    bool contains(const std::string& k) const {
        if (t_ != Type::Object) return false;
        for (auto& kv : obj_) if (kv.first == k) return true;
        return false;
    }
    const Json& at(const std::string& k) const {
        if (t_ == Type::Object) for (auto& kv : obj_) if (kv.first == k) return kv.second;
        throw std::runtime_error("json: missing key '" + k + "'");
    }
    Json& set(const std::string& k, Json v) {
        if (t_ == Type::Null) t_ = Type::Object;
        if (t_ != Type::Object) throw std::runtime_error("json: set on non-object");
        for (auto& kv : obj_) if (kv.first == k) { kv.second = std::move(v); return kv.second; }
        obj_.emplace_back(k, std::move(v));
        return obj_.back().second;
    }
    void push(Json v) {
        if (t_ == Type::Null) t_ = Type::Array;
        if (t_ != Type::Array) throw std::runtime_error("json: push on non-array");
        arr_.push_back(std::move(v));
    }

    double value(const std::string& k, double def) const { return contains(k) ? at(k).as_number() : def; }
    bool value_bool(const std::string& k, bool def) const { return contains(k) ? at(k).as_bool() : def; }
    std::string value_str(const std::string& k, const std::string& def) const {
        return contains(k) ? at(k).as_string() : def;
    }

    static Json parse(const char* text) {
        if (!text) throw std::runtime_error("json: null text");
        Parser p{text, text + std::strlen(text)};
        p.ws();
        Json v = p.value(0);
        p.ws();
        if (p.s != p.e) throw std::runtime_error("json: trailing characters");
        return v;
    }

    std::string dump() const {
        std::string out;
        dump_to(out);
        return out;
    }

    void dump_to(std::string& out) const {
        switch (t_) {
            case Type::Null: out += "null"; break;
            case Type::Bool: out += b_ ? "true" : "false"; break;
            case Type::Number: {
                char buf[64];
                double r = (double)(long long)num_;
                if (r == num_ && num_ > -9.0e15 && num_ < 9.0e15) std::snprintf(buf, sizeof buf, "%lld", (long long)num_);
                else std::snprintf(buf, sizeof buf, "%.17g", num_);
                out += buf;
                break;
            }
            case Type::String: dump_str(out, str_); break;
            case Type::Array: {
                out += '[';
                for (size_t i = 0; i < arr_.size(); ++i) { if (i) out += ','; arr_[i].dump_to(out); }
                out += ']';
                break;
            }
            case Type::Object: {
                out += '{';
                for (size_t i = 0; i < obj_.size(); ++i) {
                    if (i) out += ',';
                    dump_str(out, obj_[i].first);
                    out += ':';
                    obj_[i].second.dump_to(out);
                }
                out += '}';
                break;
            }
        }
    }

private:
    static void dump_str(std::string& out, const std::string& s) {
        out += '"';
        for (char c : s) {
            if (c == '"' || c == '\\') { out += '\\'; out += c; }
            else if ((unsigned char)c < 0x20) { char b[8]; std::snprintf(b, sizeof b, "\\u%04x", c); out += b; }
            else out += c;
        }
        out += '"';
    }

    struct Parser {
        const char* s;
        const char* e;
        void ws() { while (s < e && (*s == ' ' || *s == '\t' || *s == '\n' || *s == '\r')) ++s; }
        [[noreturn]] void fail(const char* what) { throw std::runtime_error(std::string("json: ") + what); }
        Json value(int depth) {
            if (depth > 64) fail("nesting too deep");
            if (s >= e) fail("unexpected end");
            char c = *s;
            if (c == '{') return obj(depth);
            if (c == '[') return arr(depth);
            if (c == '"') return Json::string(str());
            if (c == 't' && e - s >= 4 && !std::strncmp(s, "true", 4)) { s += 4; return Json::boolean(true); }
            if (c == 'f' && e - s >= 5 && !std::strncmp(s, "false", 5)) { s += 5; return Json::boolean(false); }
            if (c == 'n' && e - s >= 4 && !std::strncmp(s, "null", 4)) { s += 4; return Json(); }
            return num();
        }
        Json num() {
            char* end = nullptr;
            double v = std::strtod(s, &end);
            if (end == s || end > e) fail("bad number");
            s = end;
            return Json::number(v);
        }
        std::string str() {
            ++s;  // opening quote
            std::string out;
            while (s < e && *s != '"') {
                char c = *s++;
                if (c == '\\') {
                    if (s >= e) fail("bad escape");
                    char d = *s++;
                    switch (d) {
                        case '"': out += '"'; break;
                        case '\\': out += '\\'; break;
                        case '/': out += '/'; break;
                        case 'b': out += '\b'; break;
                        case 'f': out += '\f'; break;
                        case 'n': out += '\n'; break;
                        case 'r': out += '\r'; break;
                        case 't': out += '\t'; break;
                        case 'u': {
                            if (e - s < 4) fail("bad unicode escape");
                            unsigned cp = (unsigned)std::strtoul(std::string(s, 4).c_str(), nullptr, 16);
                            s += 4;
                            if (cp < 0x80) out += (char)cp;
                            else if (cp < 0x800) { out += (char)(0xC0 | (cp >> 6)); out += (char)(0x80 | (cp & 0x3F)); }
                            else { out += (char)(0xE0 | (cp >> 12)); out += (char)(0x80 | ((cp >> 6) & 0x3F)); out += (char)(0x80 | (cp & 0x3F)); }
                            break;
                        }
                        default: fail("bad escape");
                    }
                } else {
                    out += c;
                }
            }
            if (s >= e) fail("unterminated string");
            ++s;
            return out;
        }
        Json arr(int depth) {
            ++s;
            Json a = Json::array();
            ws();
            if (s < e && *s == ']') { ++s; return a; }
            for (;;) {
                ws();
                a.push(value(depth + 1));
                ws();
                if (s < e && *s == ',') { ++s; continue; }
                if (s < e && *s == ']') { ++s; return a; }
                fail("expected , or ]");
            }
        }
        Json obj(int depth) {
            ++s;
            Json o = Json::object();
            ws();
            if (s < e && *s == '}') { ++s; return o; }
            for (;;) {
                ws();
                if (s >= e || *s != '"') fail("expected key");
                std::string k = str();
                ws();
                if (s >= e || *s != ':') fail("expected :");
                ++s;
                ws();
                o.set(k, value(depth + 1));
                ws();
                if (s < e && *s == ',') { ++s; continue; }
                if (s < e && *s == '}') { ++s; return o; }
                fail("expected , or }");
            }
        }
    };

    Type t_ = Type::Null;
    bool b_ = false;
    double num_ = 0.0;
    std::string str_;
    std::vector<Json> arr_;
    std::vector<std::pair<std::string, Json>> obj_;
};

}  // namespace nlod
