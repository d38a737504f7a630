// toml_lite.h — the subset of TOML the reference's input files use:
// key = value with basic/literal strings, integers, floats (incl. 1e7, inf,
// nan), booleans, arrays, inline tables; [table] and [a.b] headers; dotted
// keys; comments.  Array-of-tables headers are rejected.
#pragma once

#include <map>
#include <memory>
#include <optional>
#include <stdexcept>
#include <string>
#include <vector>

namespace tomllite {

struct Value;
using Table = std::map<std::string, Value>;

struct Value {
    enum Type { NONE, STRING, INTEGER, FLOAT, BOOLEAN, ARRAY, TABLE } type = NONE;
    std::string s;
    long long i = 0;
    double f = 0.0;
    bool b = false;
    std::vector<Value> arr;
    std::shared_ptr<Table> tbl;

    bool is_number() const { return type == INTEGER || type == FLOAT; }
    // toml++-like permissive conversions used by the reference's getters
    std::optional<double> as_double() const {
        if(type == FLOAT) return f;
        if(type == INTEGER) return (double) i;
        return std::nullopt;
    }
    std::optional<long long> as_integer() const {
        if(type == INTEGER) return i;
        if(type == FLOAT && f == (double) (long long) f) return (long long) f;
        return std::nullopt;
    }
    std::optional<bool> as_bool() const {
        if(type == BOOLEAN) return b;
        return std::nullopt;
    }
    std::optional<std::string> as_string() const {
        if(type == STRING) return s;
        return std::nullopt;
    }
};

struct ParseError : std::runtime_error {
    using std::runtime_error::runtime_error;
};

// Parse a whole document; throws ParseError with a line number.
Table parse(const std::string &text);
Table parse_file(const std::string &path);

// Node at a dotted path ("a.b.c"), or nullptr.
const Value *find(const Table &root, const std::string &path);

}  // namespace tomllite
