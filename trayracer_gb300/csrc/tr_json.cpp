// Recursive-descent JSON reader (RFC 8259) with a nesting limit.
#include "tr_json.h"

#include <cstdlib>
#include <cstring>

namespace tr {
namespace json {

namespace {

constexpr int kMaxDepth = 256;

struct Parser {
    const std::string& s;
    size_t i = 0;
    std::string err;

    explicit Parser(const std::string& text) : s(text) {}

    bool fail(const std::string& what)
    {
        if (err.empty())
            err = what + " at byte " + std::to_string(i);
        return false;
    }

    void ws()
    {
        while (i < s.size() && (s[i] == ' ' || s[i] == '\t' || s[i] == '\n' || s[i] == '\r'))
            ++i;
    }

    bool literal(const char* word, Value& v, Value::Type t, bool b)
    {
        const size_t n = std::strlen(word);
        if (s.compare(i, n, word) != 0)
            return fail("unexpected token");
        i += n;
        v.type = t;
        v.b = b;
        return true;
    }

    static void put_utf8(std::string& out, uint32_t cp)
    {
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

    bool hex4(uint32_t& cp)
    {
        if (i + 4 > s.size())
            return fail("truncated \\u escape");
        cp = 0;
        for (int k = 0; k < 4; ++k) {
            const char c = s[i++];
            cp <<= 4;
            if (c >= '0' && c <= '9')
                cp |= uint32_t(c - '0');
            else if (c >= 'a' && c <= 'f')
                cp |= uint32_t(c - 'a' + 10);
            else if (c >= 'A' && c <= 'F')
                cp |= uint32_t(c - 'A' + 10);
            else
                return fail("bad \\u escape");
        }
        return true;
    }

    bool string(std::string& out)
    {
        ++i;  // opening quote
        while (true) {
            if (i >= s.size())
                return fail("unterminated string");
            const unsigned char c = static_cast<unsigned char>(s[i++]);
            if (c == '"')
                return true;
            if (c < 0x20)
                return fail("control character in string");
            if (c != '\\') {
                out += char(c);
                continue;
            }
            if (i >= s.size())
                return fail("unterminated escape");
            const char e = s[i++];
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
                uint32_t cp;
                if (!hex4(cp))
                    return false;
                if (cp >= 0xD800 && cp <= 0xDBFF) {
                    uint32_t lo;
                    if (i + 2 > s.size() || s[i] != '\\' || s[i + 1] != 'u')
                        return fail("unpaired surrogate");
                    i += 2;
                    if (!hex4(lo) || lo < 0xDC00 || lo > 0xDFFF)
                        return fail("unpaired surrogate");
                    cp = 0x10000 + ((cp - 0xD800) << 10) + (lo - 0xDC00);
                } else if (cp >= 0xDC00 && cp <= 0xDFFF) {
                    return fail("unpaired surrogate");
                }
                put_utf8(out, cp);
                break;
            }
            default:
                return fail("bad escape");
            }
        }
    }

    bool number(Value& v)
    {
        const size_t start = i;
        bool integral = true;
        if (s[i] == '-')
            ++i;
        if (i >= s.size() || !(s[i] >= '0' && s[i] <= '9'))
            return fail("bad number");
        if (s[i] == '0')
            ++i;
        else
            while (i < s.size() && s[i] >= '0' && s[i] <= '9')
                ++i;
        if (i < s.size() && s[i] == '.') {
            integral = false;
            ++i;
            if (i >= s.size() || !(s[i] >= '0' && s[i] <= '9'))
                return fail("bad number");
            while (i < s.size() && s[i] >= '0' && s[i] <= '9')
                ++i;
        }
        if (i < s.size() && (s[i] == 'e' || s[i] == 'E')) {
            integral = false;
            ++i;
            if (i < s.size() && (s[i] == '+' || s[i] == '-'))
                ++i;
            if (i >= s.size() || !(s[i] >= '0' && s[i] <= '9'))
                return fail("bad number");
            while (i < s.size() && s[i] >= '0' && s[i] <= '9')
                ++i;
        }
        const std::string tok = s.substr(start, i - start);
        v.type = Value::Type::Number;
        v.num = std::strtod(tok.c_str(), nullptr);
        v.integral = integral;
        return true;
    }

    bool value(Value& v, int depth)
    {
        if (depth > kMaxDepth)
            return fail("nesting too deep");
        ws();
        if (i >= s.size())
            return fail("unexpected end");
        const char c = s[i];
        if (c == '{') {
            ++i;
            v.type = Value::Type::Object;
            ws();
            if (i < s.size() && s[i] == '}') {
                ++i;
                return true;
            }
            while (true) {
                ws();
                if (i >= s.size() || s[i] != '"')
                    return fail("expected member name");
                std::string key;
                if (!string(key))
                    return false;
                ws();
                if (i >= s.size() || s[i] != ':')
                    return fail("expected ':'");
                ++i;
                Value m;
                if (!value(m, depth + 1))
                    return false;
                v.members.emplace_back(std::move(key), std::move(m));
                ws();
                if (i < s.size() && s[i] == ',') {
                    ++i;
                    continue;
                }
                if (i < s.size() && s[i] == '}') {
                    ++i;
                    return true;
                }
                return fail("expected ',' or '}'");
            }
        }
        if (c == '[') {
            ++i;
            v.type = Value::Type::Array;
            ws();
            if (i < s.size() && s[i] == ']') {
                ++i;
                return true;
            }
            while (true) {
                Value item;
                if (!value(item, depth + 1))
                    return false;
                v.items.push_back(std::move(item));
                ws();
                if (i < s.size() && s[i] == ',') {
                    ++i;
                    continue;
                }
                if (i < s.size() && s[i] == ']') {
                    ++i;
                    return true;
                }
                return fail("expected ',' or ']'");
            }
        }
        if (c == '"') {
            v.type = Value::Type::String;
            return string(v.str);
        }
        if (c == 't')
            return literal("true", v, Value::Type::Bool, true);
        if (c == 'f')
            return literal("false", v, Value::Type::Bool, false);
        if (c == 'n')
            return literal("null", v, Value::Type::Null, false);
        if (c == '-' || (c >= '0' && c <= '9'))
            return number(v);
        return fail("unexpected character");
    }
};

}  // namespace

bool parse(const std::string& text, Value& out, std::string& error)
{
    Parser p(text);
    out = Value{};
    if (!p.value(out, 0)) {
        error = p.err;
        return false;
    }
    p.ws();
    if (p.i != text.size()) {
        error = "trailing characters at byte " + std::to_string(p.i);
        return false;
    }
    return true;
}

}  // namespace json
}  // namespace tr
