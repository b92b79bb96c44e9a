// json_lite.hpp — reader for the flat JSON objects of an experiment directory
// (ModelParams.json, ParticleParams.json): one object whose values are numbers,
// booleans, strings or null. Nested objects/arrays are parsed and skipped.
#pragma once

#include <cctype>
#include <cstdlib>
#include <map>
#include <stdexcept>
#include <string>

namespace rrsph {

struct JsonValue {
    enum Kind { Number, Bool, String, Null, Other } kind = Null;
    double number = 0;
    bool boolean = false;
    std::string text;
};

class JsonObject {
public:
    static JsonObject parse(const std::string& src) {
        JsonObject obj;
        size_t i = 0;
        skip_ws(src, i);
        expect(src, i, '{');
        skip_ws(src, i);
        if (peek(src, i) == '}') return obj;
        for (;;) {
            skip_ws(src, i);
            std::string key = parse_string(src, i);
            skip_ws(src, i);
            expect(src, i, ':');
            skip_ws(src, i);
            obj.values_[key] = parse_value(src, i);
            skip_ws(src, i);
            const char c = peek(src, i);
            if (c == ',') { i++; continue; }
            if (c == '}') { i++; break; }
            throw std::runtime_error("json: expected ',' or '}' at offset " + std::to_string(i));
        }
        return obj;
    }
    bool contains(const std::string& k) const { return values_.count(k) != 0; }
    const JsonValue& at(const std::string& k) const {
        auto it = values_.find(k);
        if (it == values_.end()) throw std::runtime_error("json: missing key " + k);
        return it->second;
    }
    double number(const std::string& k) const {
        const JsonValue& v = at(k);
        if (v.kind == JsonValue::Number) return v.number;
        if (v.kind == JsonValue::Bool) return v.boolean ? 1.0 : 0.0;
        throw std::runtime_error("json: key " + k + " is not a number");
    }

private:
    std::map<std::string, JsonValue> values_;

    static char peek(const std::string& s, size_t i) { return i < s.size() ? s[i] : '\0'; }
    static void skip_ws(const std::string& s, size_t& i) {
        while (i < s.size() && std::isspace((unsigned char)s[i])) i++;
    }
    static void expect(const std::string& s, size_t& i, char c) {
        if (peek(s, i) != c)
            throw std::runtime_error(std::string("json: expected '") + c + "' at offset " + std::to_string(i));
        i++;
    }
    static std::string parse_string(const std::string& s, size_t& i) {
        expect(s, i, '"');
        std::string out;
        while (i < s.size() && s[i] != '"') {
            if (s[i] == '\\' && i + 1 < s.size()) {
                i++;
                switch (s[i]) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': out += '?'; i += 4; break;
                default: out += s[i]; break;
                }
                i++;
            } else {
                out += s[i++];
            }
        }
        expect(s, i, '"');
        return out;
    }
    static void skip_compound(const std::string& s, size_t& i) {
        int depth = 0;
        do {
            const char c = peek(s, i);
            if (c == '\0') throw std::runtime_error("json: unterminated value");
            if (c == '"') { parse_string(s, i); continue; }
            if (c == '{' || c == '[') depth++;
            if (c == '}' || c == ']') depth--;
            i++;
        } while (depth > 0);
    }
    static JsonValue parse_value(const std::string& s, size_t& i) {
        JsonValue v;
        const char c = peek(s, i);
        if (c == '"') {
            v.kind = JsonValue::String;
            v.text = parse_string(s, i);
        } else if (c == '{' || c == '[') {
            v.kind = JsonValue::Other;
            skip_compound(s, i);
        } else if (s.compare(i, 4, "true") == 0) {
            v.kind = JsonValue::Bool; v.boolean = true; i += 4;
        } else if (s.compare(i, 5, "false") == 0) {
            v.kind = JsonValue::Bool; v.boolean = false; i += 5;
        } else if (s.compare(i, 4, "null") == 0) {
            v.kind = JsonValue::Null; i += 4;
        } else {
            const char* begin = s.c_str() + i;
            char* end = nullptr;
            v.number = std::strtod(begin, &end);
            if (end == begin) throw std::runtime_error("json: bad value at offset " + std::to_string(i));
            v.kind = JsonValue::Number;
            i += (size_t)(end - begin);
        }
        return v;
    }
};

}  // namespace rrsph
