// json.h -- a small JSON reader for training_config.json and JSON sites files.
#pragma once

#include <cctype>
#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace sadcli {

struct Json {
    enum Kind { Null, Bool, Number, String, Array, Object } kind = Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::map<std::string, Json> obj;

    bool has(const std::string& k) const { return kind == Object && obj.count(k) != 0; }
    const Json& at(const std::string& k) const {
        auto it = obj.find(k);
        if (kind != Object || it == obj.end()) throw std::runtime_error("missing JSON key " + k);
        return it->second;
    }
    double number() const {
        if (kind == Number) return num;
        if (kind == Bool) return b ? 1.0 : 0.0;
        throw std::runtime_error("JSON value is not a number");
    }
};

class JsonParser {
  public:
    explicit JsonParser(const std::string& text) : s_(text) {}
    Json parse() {
        Json v = value();
        ws();
        if (i_ != s_.size()) fail("trailing characters");
        return v;
    }

  private:
    const std::string& s_;
    size_t i_ = 0;

    [[noreturn]] void fail(const char* what) {
        throw std::runtime_error(std::string("JSON: ") + what + " at offset " + std::to_string(i_));
    }
    void ws() {
        while (i_ < s_.size() && std::isspace(static_cast<unsigned char>(s_[i_]))) ++i_;
    }
    bool eat(char c) {
        ws();
        if (i_ < s_.size() && s_[i_] == c) {
            ++i_;
            return true;
        }
        return false;
    }
    std::string string() {
        if (!eat('"')) fail("expected string");
        std::string out;
        while (i_ < s_.size() && s_[i_] != '"') {
            char c = s_[i_++];
            if (c == '\\' && i_ < s_.size()) {
                char e = s_[i_++];
                switch (e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case 'r': out += '\r'; break;
                    case 'b': out += '\b'; break;
                    case 'f': out += '\f'; break;
                    case 'u': i_ += 4; out += '?'; break;  // escapes beyond ASCII are not needed here
                    default: out += e;
                }
            } else {
                out += c;
            }
        }
        if (i_ >= s_.size()) fail("unterminated string");
        ++i_;
        return out;
    }
    Json value() {
        ws();
        if (i_ >= s_.size()) fail("unexpected end");
        Json v;
        char c = s_[i_];
        if (c == '{') {
            ++i_;
            v.kind = Json::Object;
            if (eat('}')) return v;
            do {
                std::string k = string();
                if (!eat(':')) fail("expected ':'");
                v.obj[k] = value();
            } while (eat(','));
            if (!eat('}')) fail("expected '}'");
        } else if (c == '[') {
            ++i_;
            v.kind = Json::Array;
            if (eat(']')) return v;
            do v.arr.push_back(value());
            while (eat(','));
            if (!eat(']')) fail("expected ']'");
        } else if (c == '"') {
            v.kind = Json::String;
            v.str = string();
        } else if (s_.compare(i_, 4, "true") == 0) {
            i_ += 4;
            v.kind = Json::Bool;
            v.b = true;
        } else if (s_.compare(i_, 5, "false") == 0) {
            i_ += 5;
            v.kind = Json::Bool;
        } else if (s_.compare(i_, 4, "null") == 0) {
            i_ += 4;
        } else {
            const char* start = s_.c_str() + i_;
            char* end = nullptr;
            v.num = std::strtod(start, &end);
            if (end == start) fail("unexpected character");
            i_ += static_cast<size_t>(end - start);
            v.kind = Json::Number;
        }
        return v;
    }
};

}  // namespace sadcli
