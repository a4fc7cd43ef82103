// A small JSON document model, reader and writer for simulation state files
// (objects keep their key order). Numbers keep their text so integers of any
// width and floats round-trip exactly.
#pragma once

#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace flamegpu {
namespace detail {
namespace json {

struct Value {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    std::string text;                                  // number text or string value
    std::vector<Value> items;                          // array
    std::vector<std::pair<std::string, Value>> fields;  // object, in order
    const Value* find(const std::string& k) const {
        for (const auto& f : fields)
            if (f.first == k) return &f.second;
        return nullptr;
    }
    double number() const { return std::strtod(text.c_str(), nullptr); }
    long long integer() const { return std::strtoll(text.c_str(), nullptr, 10); }
    unsigned long long uinteger() const { return std::strtoull(text.c_str(), nullptr, 10); }
};

class Parser {
 public:
    explicit Parser(const std::string& s) : s_(s) {}
    Value parse() {
        Value v = value();
        ws();
        if (p_ != s_.size()) fail("trailing characters");
        return v;
    }

 private:
    [[noreturn]] void fail(const char* what) {
        throw std::runtime_error(std::string("JSON: ") + what + " at offset " + std::to_string(p_));
    }
    void ws() {
        while (p_ < s_.size() && (s_[p_] == ' ' || s_[p_] == '\n' || s_[p_] == '\r' || s_[p_] == '\t')) ++p_;
    }
    bool eat(char c) {
        ws();
        if (p_ < s_.size() && s_[p_] == c) {
            ++p_;
            return true;
        }
        return false;
    }
    void expect(char c) {
        if (!eat(c)) fail("unexpected character");
    }
    std::string str() {
        expect('"');
        std::string out;
        while (p_ < s_.size() && s_[p_] != '"') {
            char c = s_[p_++];
            if (c == '\\') {
                if (p_ >= s_.size()) fail("bad escape");
                const char e = s_[p_++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': {
                        if (p_ + 4 > s_.size()) fail("bad \\u escape");
                        const unsigned cp = static_cast<unsigned>(std::strtoul(s_.substr(p_, 4).c_str(), nullptr, 16));
                        p_ += 4;
                        if (cp < 0x80) out += static_cast<char>(cp);
                        else if (cp < 0x800) {
                            out += static_cast<char>(0xC0 | (cp >> 6));
                            out += static_cast<char>(0x80 | (cp & 0x3F));
                        } else {
                            out += static_cast<char>(0xE0 | (cp >> 12));
                            out += static_cast<char>(0x80 | ((cp >> 6) & 0x3F));
                            out += static_cast<char>(0x80 | (cp & 0x3F));
                        }
                        break;
                    }
                    default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (p_ >= s_.size()) fail("unterminated string");
        ++p_;
        return out;
    }
    Value value() {
        ws();
        if (p_ >= s_.size()) fail("unexpected end");
        Value v;
        const char c = s_[p_];
        if (c == '{') {
            ++p_;
            v.kind = Value::Object;
            if (eat('}')) return v;
            do {
                ws();
                std::string k = str();
                expect(':');
                v.fields.emplace_back(std::move(k), value());
            } while (eat(','));
            expect('}');
        } else if (c == '[') {
            ++p_;
            v.kind = Value::Array;
            if (eat(']')) return v;
            do {
                v.items.push_back(value());
            } while (eat(','));
            expect(']');
        } else if (c == '"') {
            v.kind = Value::String;
            v.text = str();
        } else if (s_.compare(p_, 4, "true") == 0) {
            v.kind = Value::Bool;
            v.b = true;
            p_ += 4;
        } else if (s_.compare(p_, 5, "false") == 0) {
            v.kind = Value::Bool;
            p_ += 5;
        } else if (s_.compare(p_, 4, "null") == 0) {
            p_ += 4;
        } else {
            const size_t b = p_;
            while (p_ < s_.size() && (std::strchr("+-0123456789.eE", s_[p_]) != nullptr)) ++p_;
            if (b == p_) fail("unexpected character");
            v.kind = Value::Number;
            v.text = s_.substr(b, p_ - b);
        }
        return v;
    }
    const std::string& s_;
    size_t p_ = 0;
};

/** Streaming writer with two-space indentation. */
class Writer {
 public:
    explicit Writer(std::FILE* f) : f_(f) {}
    void begin_object() { open('{'); }
    void end_object() { close('}'); }
    void begin_array() { open('['); }
    void end_array() { close(']'); }
    void key(const std::string& k) {
        sep();
        indent();
        quoted(k);
        std::fputs(": ", f_);
        after_key_ = true;
    }
    void raw(const std::string& text) {
        value_prefix();
        std::fputs(text.c_str(), f_);
    }
    void string(const std::string& s) {
        value_prefix();
        quoted(s);
    }

 private:
    void quoted(const std::string& s) {
        std::fputc('"', f_);
        for (char c : s) {
            if (c == '"' || c == '\\') {
                std::fputc('\\', f_);
                std::fputc(c, f_);
            } else if (c == '\n') {
                std::fputs("\\n", f_);
            } else {
                std::fputc(c, f_);
            }
        }
        std::fputc('"', f_);
    }
    void sep() {
        if (!first_.empty() && !first_.back()) std::fputc(',', f_);
        if (!first_.empty()) first_.back() = false;
        if (!first_.empty()) std::fputc('\n', f_);
    }
    void indent() {
        for (size_t i = 0; i < first_.size(); ++i) std::fputs("  ", f_);
    }
    void value_prefix() {
        if (after_key_) {
            after_key_ = false;
            return;
        }
        sep();
        indent();
    }
    void open(char c) {
        value_prefix();
        std::fputc(c, f_);
        first_.push_back(true);
    }
    void close(char c) {
        const bool empty = first_.back();
        first_.pop_back();
        if (!empty) {
            std::fputc('\n', f_);
            indent();
        }
        std::fputc(c, f_);
    }
    std::FILE* f_;
    std::vector<bool> first_;
    bool after_key_ = false;
};

}  // namespace json
}  // namespace detail
}  // namespace flamegpu
