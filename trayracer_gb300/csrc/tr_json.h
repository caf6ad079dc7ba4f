// Minimal JSON reader (RFC 8259) for scene files: a DOM of null, bool,
// number, string, array and object values. Objects keep their members in file
// order; a lookup returns the first member of that name.
#pragma once

#include <cstdint>
#include <memory>
#include <string>
#include <utility>
#include <vector>

namespace tr {
namespace json {

struct Value {
    enum class Type { Null, Bool, Number, String, Array, Object };
    Type type = Type::Null;
    bool b = false;
    double num = 0.0;
    bool integral = false;   // the number was written without fraction or exponent
    std::string str;
    std::vector<Value> items;                           // array
    std::vector<std::pair<std::string, Value>> members; // object

    bool is_number() const { return type == Type::Number; }
    bool is_string() const { return type == Type::String; }
    bool is_array() const { return type == Type::Array; }
    bool is_object() const { return type == Type::Object; }
    bool is_bool() const { return type == Type::Bool; }
    // first member named key, or null
    const Value* find(const std::string& key) const
    {
        if (type != Type::Object)
            return nullptr;
        for (const auto& m : members)
            if (m.first == key)
                return &m.second;
        return nullptr;
    }
};

// Parses text; on failure returns false with a message naming the byte offset.
bool parse(const std::string& text, Value& out, std::string& error);

}  // namespace json
}  // namespace tr
