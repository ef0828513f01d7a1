// Minimal YAML reader for nanogi scene files.
//
// The reference parses scenes with yaml-cpp (include/nanogi/rt.hpp:1525). Scene files
// (schema.yml:33-334) only use block mappings, block sequences ("- "), flow sequences of
// scalars ("[L, D]", "[0.5, 1, 2]"), plain / quoted scalars and comments, so this reader
// supports exactly that subset and reports anything else as a parse error with a line
// number instead of guessing.
#pragma once

#include <map>
#include <memory>
#include <stdexcept>
#include <string>
#include <vector>

namespace ngi {

struct YamlError : std::runtime_error {
    explicit YamlError(const std::string& m) : std::runtime_error(m) {}
};

class YamlNode {
public:
    enum class Kind { Null, Scalar, Sequence, Mapping };

    Kind kind = Kind::Null;
    std::string scalar;
    std::vector<std::shared_ptr<YamlNode>> seq;
    std::vector<std::pair<std::string, std::shared_ptr<YamlNode>>> map;  // insertion order
    int line = 0;

    bool IsNull() const { return kind == Kind::Null; }
    bool IsScalar() const { return kind == Kind::Scalar; }
    bool IsSequence() const { return kind == Kind::Sequence; }
    bool IsMapping() const { return kind == Kind::Mapping; }
    size_t size() const { return kind == Kind::Sequence ? seq.size() : (kind == Kind::Mapping ? map.size() : 0); }

    // Mapping lookup; returns a shared Null node when absent (mirrors yaml-cpp's falsy node).
    const YamlNode& operator[](const std::string& key) const;
    const YamlNode& operator[](size_t i) const;
    bool Has(const std::string& key) const;

    std::string AsString() const;
    double AsDouble() const;
    int AsInt() const;
    bool AsBool() const;
};

// Parses a whole document. Throws YamlError on malformed input.
std::shared_ptr<YamlNode> YamlParse(const std::string& text);
std::shared_ptr<YamlNode> YamlLoadFile(const std::string& path);

}  // namespace ngi
