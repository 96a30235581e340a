// Minimal JSON document reader for the schema-6 transport configuration
// (transport_physics.json) and the RREATBL container headers.  Only what the
// table loader needs: objects, arrays, strings, numbers, booleans, null.
// Numbers keep their source text so callers can parse them with strtod
// exactly as the reference's text scanner does (native_amrex_rrea/src/
// RreaInteractionTables.cpp:161-337 reads values as text, then converts).
#pragma once

#include <cstdlib>
#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace rrea_host {

struct JsonValue {
    enum class Kind { Null, Bool, Number, String, Array, Object };
    Kind kind = Kind::Null;
    bool boolean = false;
    std::string text;  // string contents, or number source text
    std::vector<JsonValue> items;
    std::vector<std::pair<std::string, JsonValue>> members;

    bool is_object() const { return kind == Kind::Object; }
    bool is_array() const { return kind == Kind::Array; }

    JsonValue const* find(std::string const& key) const
    {
        for (auto const& m : members) {
            if (m.first == key) {
                return &m.second;
            }
        }
        return nullptr;
    }
    JsonValue const& at(std::string const& key) const
    {
        JsonValue const* v = find(key);
        if (!v) {
            throw std::runtime_error("json: missing key '" + key + "'");
        }
        return *v;
    }
    std::string str(std::string const& key) const
    {
        JsonValue const& v = at(key);
        if (v.kind != Kind::String && v.kind != Kind::Number) {
            throw std::runtime_error("json: key '" + key + "' is not a string");
        }
        return v.text;
    }
    std::string str_or(std::string const& key, std::string const& fallback) const
    {
        JsonValue const* v = find(key);
        if (!v || (v->kind != Kind::String && v->kind != Kind::Number)) {
            return fallback;
        }
        return v->text;
    }
    double num() const
    {
        if (kind == Kind::Number || kind == Kind::String) {
            char* end = nullptr;
            double const value = std::strtod(text.c_str(), &end);
            if (end == text.c_str()) {
                throw std::runtime_error("json: not a number: " + text);
            }
            return value;
        }
        throw std::runtime_error("json: value is not numeric");
    }
    double num_or(std::string const& key, double fallback) const
    {
        JsonValue const* v = find(key);
        return v ? v->num() : fallback;
    }
    bool bool_or(std::string const& key, bool fallback) const
    {
        JsonValue const* v = find(key);
        if (!v) {
            return fallback;
        }
        if (v->kind == Kind::Bool) {
            return v->boolean;
        }
        if (v->kind == Kind::String) {
            return v->text == "true" || v->text == "1";
        }
        return fallback;
    }
};

class JsonParser {
public:
    explicit JsonParser(std::string const& text) : m_text(text) {}

    JsonValue parse()
    {
        JsonValue v = value();
        skip();
        if (m_pos != m_text.size()) {
            throw std::runtime_error("json: trailing characters");
        }
        return v;
    }

private:
    std::string const& m_text;
    std::size_t m_pos = 0;

    void skip()
    {
        while (m_pos < m_text.size()
               && (m_text[m_pos] == ' ' || m_text[m_pos] == '\n'
                   || m_text[m_pos] == '\r' || m_text[m_pos] == '\t')) {
            ++m_pos;
        }
    }
    char peek()
    {
        skip();
        if (m_pos >= m_text.size()) {
            throw std::runtime_error("json: unexpected end");
        }
        return m_text[m_pos];
    }
    void expect(char c)
    {
        if (peek() != c) {
            throw std::runtime_error(std::string("json: expected '") + c + "'");
        }
        ++m_pos;
    }
    std::string string_body()
    {
        expect('"');
        std::string out;
        while (m_pos < m_text.size() && m_text[m_pos] != '"') {
            char c = m_text[m_pos++];
            if (c == '\\' && m_pos < m_text.size()) {
                char e = m_text[m_pos++];
                switch (e) {
                case 'n': out.push_back('\n'); break;
                case 't': out.push_back('\t'); break;
                case 'r': out.push_back('\r'); break;
                case 'b': out.push_back('\b'); break;
                case 'f': out.push_back('\f'); break;
                case 'u': {
                    // Table headers are ASCII; keep the escape verbatim.
                    out += "\\u";
                    break;
                }
                default: out.push_back(e); break;
                }
            } else {
                out.push_back(c);
            }
        }
        if (m_pos >= m_text.size()) {
            throw std::runtime_error("json: unterminated string");
        }
        ++m_pos;
        return out;
    }
    JsonValue value()
    {
        char const c = peek();
        JsonValue v;
        if (c == '{') {
            v.kind = JsonValue::Kind::Object;
            ++m_pos;
            if (peek() == '}') {
                ++m_pos;
                return v;
            }
            for (;;) {
                std::string key = string_body();
                expect(':');
                v.members.emplace_back(std::move(key), value());
                char const d = peek();
                ++m_pos;
                if (d == '}') {
                    break;
                }
                if (d != ',') {
                    throw std::runtime_error("json: expected ',' in object");
                }
            }
            return v;
        }
        if (c == '[') {
            v.kind = JsonValue::Kind::Array;
            ++m_pos;
            if (peek() == ']') {
                ++m_pos;
                return v;
            }
            for (;;) {
                v.items.push_back(value());
                char const d = peek();
                ++m_pos;
                if (d == ']') {
                    break;
                }
                if (d != ',') {
                    throw std::runtime_error("json: expected ',' in array");
                }
            }
            return v;
        }
        if (c == '"') {
            v.kind = JsonValue::Kind::String;
            v.text = string_body();
            return v;
        }
        if (m_text.compare(m_pos, 4, "true") == 0) {
            v.kind = JsonValue::Kind::Bool;
            v.boolean = true;
            m_pos += 4;
            return v;
        }
        if (m_text.compare(m_pos, 5, "false") == 0) {
            v.kind = JsonValue::Kind::Bool;
            m_pos += 5;
            return v;
        }
        if (m_text.compare(m_pos, 4, "null") == 0) {
            m_pos += 4;
            return v;
        }
        std::size_t const start = m_pos;
        while (m_pos < m_text.size()) {
            char const d = m_text[m_pos];
            if ((d >= '0' && d <= '9') || d == '-' || d == '+' || d == '.'
                || d == 'e' || d == 'E') {
                ++m_pos;
            } else {
                break;
            }
        }
        if (m_pos == start) {
            throw std::runtime_error("json: unexpected character");
        }
        v.kind = JsonValue::Kind::Number;
        v.text = m_text.substr(start, m_pos - start);
        return v;
    }
};

inline JsonValue ParseJson(std::string const& text)
{
    return JsonParser(text).parse();
}

}  // namespace rrea_host
