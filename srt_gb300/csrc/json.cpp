// json.cpp — recursive-descent JSON reader (see json.h).
#include "json.h"

#include <cstdlib>
#include <cstring>

namespace srt {
namespace {

struct Parser {
    const std::string& s;
    size_t i = 0;
    std::string err;
    int depth = 0;

    explicit Parser(const std::string& t) : s(t) {}

    bool fail(const std::string& m)
    {
        if (err.empty()) err = m + " at offset " + std::to_string(i);
        return false;
    }
    void skip()
    {
        for (;;) {
            while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r')) ++i;
            if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '/') {
                while (i < s.size() && s[i] != '\n') ++i;
                continue;
            }
            if (i + 1 < s.size() && s[i] == '/' && s[i + 1] == '*') {
                size_t e = s.find("*/", i + 2);
                i = (e == std::string::npos) ? s.size() : e + 2;
                continue;
            }
            break;
        }
    }
    bool lit(const char* w)
    {
        size_t n = std::strlen(w);
        if (s.compare(i, n, w) != 0) return false;
        i += n;
        return true;
    }
    bool string(std::string& out)
    {
        if (i >= s.size() || s[i] != '"') return fail("expected string");
        ++i;
        out.clear();
        while (i < s.size() && s[i] != '"') {
            char c = s[i++];
            if (c == '\\') {
                if (i >= s.size()) return fail("bad escape");
                char e = s[i++];
                switch (e) {
                case 'n': out += '\n'; break;
                case 't': out += '\t'; break;
                case 'r': out += '\r'; break;
                case 'b': out += '\b'; break;
                case 'f': out += '\f'; break;
                case 'u': {
                    if (i + 4 > s.size()) return fail("bad \\u escape");
                    unsigned cp = (unsigned)std::strtoul(s.substr(i, 4).c_str(), nullptr, 16);
                    i += 4;
                    if (cp < 0x80) {
                        out += (char)cp;
                    } else if (cp < 0x800) {
                        out += (char)(0xC0 | (cp >> 6));
                        out += (char)(0x80 | (cp & 0x3F));
                    } else {
                        out += (char)(0xE0 | (cp >> 12));
                        out += (char)(0x80 | ((cp >> 6) & 0x3F));
                        out += (char)(0x80 | (cp & 0x3F));
                    }
                    break;
                }
                default: out += e; break;
                }
            } else {
                out += c;
            }
        }
        if (i >= s.size()) return fail("unterminated string");
        ++i;
        return true;
    }
    bool value(Json& v)
    {
        if (++depth > 256) return fail("nesting too deep");
        skip();
        if (i >= s.size()) return fail("unexpected end");
        char c = s[i];
        bool ok = true;
        if (c == '{') {
            ++i;
            v.type = Json::Type::Object;
            skip();
            if (i < s.size() && s[i] == '}') {
                ++i;
            } else {
                for (;;) {
                    skip();
                    std::string k;
                    if (!string(k)) return false;
                    skip();
                    if (i >= s.size() || s[i] != ':') return fail("expected ':'");
                    ++i;
                    Json child;
                    if (!value(child)) return false;
                    v.obj.emplace_back(std::move(k), std::move(child));
                    skip();
                    if (i < s.size() && s[i] == ',') {
                        ++i;
                        continue;
                    }
                    if (i < s.size() && s[i] == '}') {
                        ++i;
                        break;
                    }
                    return fail("expected ',' or '}'");
                }
            }
        } else if (c == '[') {
            ++i;
            v.type = Json::Type::Array;
            skip();
            if (i < s.size() && s[i] == ']') {
                ++i;
            } else {
                for (;;) {
                    Json child;
                    if (!value(child)) return false;
                    v.arr.push_back(std::move(child));
                    skip();
                    if (i < s.size() && s[i] == ',') {
                        ++i;
                        continue;
                    }
                    if (i < s.size() && s[i] == ']') {
                        ++i;
                        break;
                    }
                    return fail("expected ',' or ']'");
                }
            }
        } else if (c == '"') {
            v.type = Json::Type::String;
            ok = string(v.str);
        } else if (lit("true")) {
            v.type = Json::Type::Bool;
            v.b = true;
        } else if (lit("false")) {
            v.type = Json::Type::Bool;
            v.b = false;
        } else if (lit("null")) {
            v.type = Json::Type::Null;
        } else if (c == '-' || (c >= '0' && c <= '9')) {
            const char* start = s.c_str() + i;
            char* end = nullptr;
            v.num = std::strtod(start, &end);
            if (end == start) return fail("bad number");
            v.type = Json::Type::Number;
            i += (size_t)(end - start);
        } else {
            return fail("unexpected character");
        }
        --depth;
        return ok;
    }
};

}  // namespace

bool Json::parse(const std::string& text, Json& out, std::string& err)
{
    Parser p(text);
    out = Json();
    if (!p.value(out)) {
        err = p.err;
        return false;
    }
    p.skip();
    if (p.i != text.size()) {
        err = "trailing characters at offset " + std::to_string(p.i);
        return false;
    }
    return true;
}

}  // namespace srt
