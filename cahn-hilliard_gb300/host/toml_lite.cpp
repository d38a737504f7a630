// toml_lite.cpp — see toml_lite.h.
#include "toml_lite.h"

#include <cctype>
#include <cmath>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace tomllite {

namespace {

struct Parser {
    const std::string &t;
    size_t p = 0;
    int line = 1;

    explicit Parser(const std::string &text) : t(text) {}

    [[noreturn]] void fail(const std::string &msg) {
        throw ParseError("TOML line " + std::to_string(line) + ": " + msg);
    }
    bool eof() const { return p >= t.size(); }
    char peek() const { return eof() ? '\0' : t[p]; }
    char get() {
        char c = t[p++];
        if(c == '\n') line++;
        return c;
    }
    void skip_ws() {
        while(!eof() && (peek() == ' ' || peek() == '\t')) p++;
    }
    void skip_comment() {
        if(peek() == '#')
            while(!eof() && peek() != '\n') p++;
    }
    // whitespace, newlines and comments (inside arrays)
    void skip_all() {
        for(;;) {
            skip_ws();
            if(peek() == '#') {
                skip_comment();
                continue;
            }
            if(peek() == '\n' || peek() == '\r') {
                get();
                continue;
            }
            break;
        }
    }
    void expect_eol() {
        skip_ws();
        skip_comment();
        if(peek() == '\r') p++;
        if(!eof() && peek() != '\n') fail("unexpected text after value");
        if(!eof()) get();
    }

    std::string bare_or_quoted_key() {
        skip_ws();
        if(peek() == '"' || peek() == '\'') return string_value();
        size_t s = p;
        while(!eof() && (std::isalnum((unsigned char) peek()) || peek() == '_' || peek() == '-')) p++;
        if(s == p) fail("expected a key");
        return t.substr(s, p - s);
    }
    std::vector<std::string> dotted_key() {
        std::vector<std::string> parts{bare_or_quoted_key()};
        for(;;) {
            skip_ws();
            if(peek() != '.') break;
            p++;
            parts.push_back(bare_or_quoted_key());
        }
        return parts;
    }

    std::string string_value() {
        char q = get();
        std::string out;
        if(q == '\'') {
            while(!eof() && peek() != '\'') {
                if(peek() == '\n') fail("newline in string");
                out += get();
            }
            if(eof()) fail("unterminated string");
            p++;
            return out;
        }
        while(!eof() && peek() != '"') {
            char c = get();
            if(c == '\n') fail("newline in string");
            if(c == '\\') {
                char e = get();
                switch(e) {
                    case 'n': out += '\n'; break;
                    case 't': out += '\t'; break;
                    case '\\': out += '\\'; break;
                    case '"': out += '"'; break;
                    case 'r': out += '\r'; break;
                    default: fail("unsupported escape");
                }
            }
            else {
                out += c;
            }
        }
        if(eof()) fail("unterminated string");
        p++;
        return out;
    }

    Value number_value() {
        size_t s = p;
        while(!eof() && (std::isalnum((unsigned char) peek()) || peek() == '+' || peek() == '-' || peek() == '.' ||
                         peek() == '_'))
            p++;
        std::string tok;
        for(size_t k = s; k < p; k++)
            if(t[k] != '_') tok += t[k];
        Value v;
        if(tok == "inf" || tok == "+inf" || tok == "-inf" || tok == "nan" || tok == "+nan" || tok == "-nan") {
            v.type = Value::FLOAT;
            v.f = (tok.find("nan") != std::string::npos) ? NAN : (tok[0] == '-' ? -INFINITY : INFINITY);
            return v;
        }
        bool is_float = tok.find_first_of(".eE") != std::string::npos &&
                        !(tok.size() > 1 && tok[0] == '0' && (tok[1] == 'x' || tok[1] == 'o' || tok[1] == 'b'));
        char *end = nullptr;
        if(is_float) {
            v.type = Value::FLOAT;
            v.f = std::strtod(tok.c_str(), &end);
        }
        else {
            v.type = Value::INTEGER;
            int base = 10;
            std::string digits = tok;
            bool neg = false;
            if(!digits.empty() && (digits[0] == '+' || digits[0] == '-')) {
                neg = digits[0] == '-';
                digits = digits.substr(1);
            }
            if(digits.size() > 2 && digits[0] == '0' && (digits[1] == 'x' || digits[1] == 'o' || digits[1] == 'b')) {
                base = digits[1] == 'x' ? 16 : (digits[1] == 'o' ? 8 : 2);
                digits = digits.substr(2);
            }
            v.i = std::strtoll(digits.c_str(), &end, base);
            if(neg) v.i = -v.i;
        }
        if(tok.empty() || (end && *end != '\0')) fail("malformed number '" + tok + "'");
        return v;
    }

    Value value() {
        skip_ws();
        char c = peek();
        Value v;
        if(c == '"' || c == '\'') {
            v.type = Value::STRING;
            v.s = string_value();
            return v;
        }
        if(t.compare(p, 4, "true") == 0) {
            p += 4;
            v.type = Value::BOOLEAN;
            v.b = true;
            return v;
        }
        if(t.compare(p, 5, "false") == 0) {
            p += 5;
            v.type = Value::BOOLEAN;
            v.b = false;
            return v;
        }
        if(c == '[') {
            p++;
            v.type = Value::ARRAY;
            skip_all();
            while(peek() != ']') {
                v.arr.push_back(value());
                skip_all();
                if(peek() == ',') {
                    p++;
                    skip_all();
                }
                else if(peek() != ']') {
                    fail("expected ',' or ']' in array");
                }
            }
            p++;
            return v;
        }
        if(c == '{') {
            p++;
            v.type = Value::TABLE;
            v.tbl = std::make_shared<Table>();
            skip_ws();
            while(peek() != '}') {
                auto key = dotted_key();
                skip_ws();
                if(get() != '=') fail("expected '=' in inline table");
                insert(*v.tbl, key, value());
                skip_ws();
                if(peek() == ',') {
                    p++;
                    skip_ws();
                }
                else if(peek() != '}') {
                    fail("expected ',' or '}' in inline table");
                }
            }
            p++;
            return v;
        }
        if(std::isdigit((unsigned char) c) || c == '+' || c == '-' || c == 'i' || c == 'n') return number_value();
        fail("unrecognised value");
    }

    Table &descend(Table &root, const std::vector<std::string> &path, size_t n) {
        Table *cur = &root;
        for(size_t k = 0; k < n; k++) {
            Value &v = (*cur)[path[k]];
            if(v.type == Value::NONE) {
                v.type = Value::TABLE;
                v.tbl = std::make_shared<Table>();
            }
            if(v.type != Value::TABLE) fail("key '" + path[k] + "' is not a table");
            cur = v.tbl.get();
        }
        return *cur;
    }

    void insert(Table &tbl, const std::vector<std::string> &key, Value v) {
        Table &parent = descend(tbl, key, key.size() - 1);
        auto &slot = parent[key.back()];
        if(slot.type != Value::NONE) fail("duplicate key '" + key.back() + "'");
        slot = std::move(v);
    }

    Table document() {
        Table root;
        std::vector<std::string> current;
        for(;;) {
            skip_all();
            if(eof()) break;
            if(peek() == '[') {
                p++;
                if(peek() == '[') fail("arrays of tables are not supported");
                current = dotted_key();
                skip_ws();
                if(get() != ']') fail("expected ']'");
                descend(root, current, current.size());
                expect_eol();
                continue;
            }
            auto key = dotted_key();
            skip_ws();
            if(get() != '=') fail("expected '='");
            Value v = value();
            insert(descend(root, current, current.size()), key, std::move(v));
            expect_eol();
        }
        return root;
    }
};

}  // namespace

Table parse(const std::string &text) {
    Parser ps(text);
    return ps.document();
}

Table parse_file(const std::string &path) {
    std::ifstream in(path);
    if(!in) throw ParseError("cannot open '" + path + "'");
    std::stringstream ss;
    ss << in.rdbuf();
    return parse(ss.str());
}

const Value *find(const Table &root, const std::string &path) {
    const Table *cur = &root;
    size_t s = 0;
    for(;;) {
        size_t dot = path.find('.', s);
        std::string part = path.substr(s, dot == std::string::npos ? std::string::npos : dot - s);
        auto it = cur->find(part);
        if(it == cur->end()) return nullptr;
        if(dot == std::string::npos) return &it->second;
        if(it->second.type != Value::TABLE) return nullptr;
        cur = it->second.tbl.get();
        s = dot + 1;
    }
}

}  // namespace tomllite
