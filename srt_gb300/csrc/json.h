// json.h — minimal JSON reader for render configurations (objects, arrays,
// strings, numbers, booleans, null; `//` and `/* */` comments are skipped,
// as the reference parses its configs with comments allowed,
// src/main/main.cu:5-17).
#pragma once

#include <map>
#include <memory>
#include <string>
#include <vector>

namespace srt {

class Json {
public:
    enum class Type { Null, Bool, Number, String, Array, Object };

    Type type = Type::Null;
    bool b = false;
    double num = 0.0;
    std::string str;
    std::vector<Json> arr;
    std::vector<std::pair<std::string, Json>> obj;

    bool is_null() const { return type == Type::Null; }
    bool is_object() const { return type == Type::Object; }
    bool is_array() const { return type == Type::Array; }
    const Json* find(const std::string& key) const
    {
        for (const auto& kv : obj)
            if (kv.first == key) return &kv.second;
        return nullptr;
    }
    bool has(const std::string& key) const { return find(key) != nullptr; }
    // j.value(key, default) of nlohmann::json
    double number(const std::string& key, double def) const
    {
        const Json* v = find(key);
        return (v && v->type == Type::Number) ? v->num : def;
    }
    bool boolean(const std::string& key, bool def) const
    {
        const Json* v = find(key);
        return (v && v->type == Type::Bool) ? v->b : def;
    }
    std::string string(const std::string& key, const std::string& def) const
    {
        const Json* v = find(key);
        return (v && v->type == Type::String) ? v->str : def;
    }
    // Parses `text`; on failure returns false and sets `err`.
    static bool parse(const std::string& text, Json& out, std::string& err);
};

}  // namespace srt
