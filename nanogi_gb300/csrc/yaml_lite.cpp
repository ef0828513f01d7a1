// Minimal YAML reader for nanogi scene files (see yaml_lite.hpp for the supported subset).
#include "yaml_lite.hpp"

#include <cerrno>
#include <cstdlib>
#include <fstream>
#include <sstream>

namespace ngi {

namespace {

const YamlNode& NullNode() {
    static const YamlNode n;
    return n;
}

struct Line {
    int indent;
    std::string text;
    int lineno;
};

std::string Trim(const std::string& s) {
    size_t b = 0, e = s.size();
    while (b < e && (s[b] == ' ' || s[b] == '\t' || s[b] == '\r')) b++;
    while (e > b && (s[e - 1] == ' ' || s[e - 1] == '\t' || s[e - 1] == '\r')) e--;
    return s.substr(b, e - b);
}

// Removes a trailing comment ('#' preceded by whitespace or at line start, outside quotes).
std::string StripComment(const std::string& s) {
    char quote = 0;
    for (size_t i = 0; i < s.size(); i++) {
        char c = s[i];
        if (quote) {
            if (c == quote) quote = 0;
            continue;
        }
        if (c == '\'' || c == '"') {
            quote = c;
            continue;
        }
        if (c == '#' && (i == 0 || s[i - 1] == ' ' || s[i - 1] == '\t')) return s.substr(0, i);
    }
    return s;
}

std::string Unquote(const std::string& raw, int lineno) {
    std::string s = Trim(raw);
    if (s.size() >= 2 && ((s.front() == '\'' && s.back() == '\'') || (s.front() == '"' && s.back() == '"'))) {
        std::string inner = s.substr(1, s.size() - 2);
        if (s.front() == '\'') {
            // '' is an escaped single quote in single-quoted scalars
            std::string out;
            for (size_t i = 0; i < inner.size(); i++) {
                if (inner[i] == '\'' && i + 1 < inner.size() && inner[i + 1] == '\'') i++;
                out.push_back(inner[i]);
            }
            return out;
        }
        std::string out;
        for (size_t i = 0; i < inner.size(); i++) {
            if (inner[i] == '\\' && i + 1 < inner.size()) {
                char n = inner[++i];
                switch (n) {
                    case 'n': out.push_back('\n'); break;
                    case 't': out.push_back('\t'); break;
                    case '\\': out.push_back('\\'); break;
                    case '"': out.push_back('"'); break;
                    default: out.push_back('\\'); out.push_back(n); break;
                }
            } else {
                out.push_back(inner[i]);
            }
        }
        return out;
    }
    if (!s.empty() && (s.front() == '\'' || s.front() == '"'))
        throw YamlError("line " + std::to_string(lineno) + ": unterminated quoted scalar");
    return s;
}

std::shared_ptr<YamlNode> MakeScalar(const std::string& raw, int lineno) {
    auto n = std::make_shared<YamlNode>();
    n->line = lineno;
    std::string t = Trim(raw);
    if (t.empty() || t == "~" || t == "null") {
        n->kind = YamlNode::Kind::Null;
        return n;
    }
    n->kind = YamlNode::Kind::Scalar;
    n->scalar = Unquote(t, lineno);
    return n;
}

// Splits the inside of a flow collection at top-level commas.
std::vector<std::string> SplitFlow(const std::string& inner, int lineno) {
    std::vector<std::string> parts;
    int depth = 0;
    char quote = 0;
    std::string cur;
    for (char c : inner) {
        if (quote) {
            cur.push_back(c);
            if (c == quote) quote = 0;
            continue;
        }
        if (c == '\'' || c == '"') { quote = c; cur.push_back(c); continue; }
        if (c == '[' || c == '{') depth++;
        if (c == ']' || c == '}') depth--;
        if (depth < 0) throw YamlError("line " + std::to_string(lineno) + ": unbalanced brackets");
        if (c == ',' && depth == 0) {
            parts.push_back(cur);
            cur.clear();
            continue;
        }
        cur.push_back(c);
    }
    if (quote || depth != 0) throw YamlError("line " + std::to_string(lineno) + ": unbalanced flow collection");
    if (!Trim(cur).empty() || !parts.empty()) parts.push_back(cur);
    return parts;
}

std::shared_ptr<YamlNode> ParseFlowOrScalar(const std::string& raw, int lineno);

std::shared_ptr<YamlNode> ParseFlow(const std::string& t, int lineno) {
    auto n = std::make_shared<YamlNode>();
    n->line = lineno;
    if (t.front() == '[') {
        if (t.back() != ']') throw YamlError("line " + std::to_string(lineno) + ": flow sequence must close on its line");
        n->kind = YamlNode::Kind::Sequence;
        for (auto& p : SplitFlow(t.substr(1, t.size() - 2), lineno)) {
            if (Trim(p).empty()) throw YamlError("line " + std::to_string(lineno) + ": empty flow sequence item");
            n->seq.push_back(ParseFlowOrScalar(p, lineno));
        }
        return n;
    }
    // '{' ... '}'
    if (t.back() != '}') throw YamlError("line " + std::to_string(lineno) + ": flow mapping must close on its line");
    n->kind = YamlNode::Kind::Mapping;
    for (auto& p : SplitFlow(t.substr(1, t.size() - 2), lineno)) {
        std::string e = Trim(p);
        size_t c = e.find(':');
        if (c == std::string::npos) throw YamlError("line " + std::to_string(lineno) + ": flow mapping item without ':'");
        n->map.emplace_back(Unquote(e.substr(0, c), lineno), ParseFlowOrScalar(e.substr(c + 1), lineno));
    }
    return n;
}

std::shared_ptr<YamlNode> ParseFlowOrScalar(const std::string& raw, int lineno) {
    std::string t = Trim(raw);
    if (!t.empty() && (t.front() == '[' || t.front() == '{')) return ParseFlow(t, lineno);
    return MakeScalar(t, lineno);
}

// Position of the mapping ':' separator (followed by space or end), outside quotes/brackets.
size_t FindKeySep(const std::string& s) {
    char quote = 0;
    int depth = 0;
    for (size_t i = 0; i < s.size(); i++) {
        char c = s[i];
        if (quote) {
            if (c == quote) quote = 0;
            continue;
        }
        if (c == '\'' || c == '"') { quote = c; continue; }
        if (c == '[' || c == '{') depth++;
        if (c == ']' || c == '}') depth--;
        if (c == ':' && depth == 0 && (i + 1 == s.size() || s[i + 1] == ' ' || s[i + 1] == '\t')) return i;
    }
    return std::string::npos;
}

bool IsSeqItem(const std::string& t) { return t == "-" || (t.size() >= 2 && t[0] == '-' && (t[1] == ' ' || t[1] == '\t')); }

class Parser {
public:
    explicit Parser(std::vector<Line> lines) : L(std::move(lines)) {}

    std::shared_ptr<YamlNode> ParseDocument() {
        if (L.empty()) return std::make_shared<YamlNode>();
        size_t i = 0;
        auto n = ParseBlock(i, L[0].indent);
        if (i != L.size())
            throw YamlError("line " + std::to_string(L[i].lineno) + ": unexpected indentation");
        return n;
    }

private:
    std::vector<Line> L;

    std::shared_ptr<YamlNode> ParseBlock(size_t& i, int indent) {
        if (i >= L.size()) return std::make_shared<YamlNode>();
        if (L[i].indent != indent)
            throw YamlError("line " + std::to_string(L[i].lineno) + ": bad indentation");
        const std::string& t = L[i].text;
        if (IsSeqItem(t)) return ParseSeq(i, indent);
        if (FindKeySep(t) != std::string::npos) return ParseMap(i, indent);
        auto n = ParseFlowOrScalar(t, L[i].lineno);
        i++;
        return n;
    }

    std::shared_ptr<YamlNode> ParseSeq(size_t& i, int indent) {
        auto n = std::make_shared<YamlNode>();
        n->kind = YamlNode::Kind::Sequence;
        n->line = L[i].lineno;
        while (i < L.size() && L[i].indent == indent && IsSeqItem(L[i].text)) {
            std::string rest = L[i].text.substr(1);
            size_t sp = 0;
            while (sp < rest.size() && (rest[sp] == ' ' || rest[sp] == '\t')) sp++;
            rest = rest.substr(sp);
            if (rest.empty()) {
                i++;
                if (i < L.size() && L[i].indent > indent) {
                    n->seq.push_back(ParseBlock(i, L[i].indent));
                } else {
                    n->seq.push_back(std::make_shared<YamlNode>());
                }
            } else {
                // "- key: value" or "- scalar": re-read the remainder as a block whose
                // indentation is the column it starts at.
                L[i].indent = indent + 1 + (int)sp;
                L[i].text = rest;
                n->seq.push_back(ParseBlock(i, L[i].indent));
            }
        }
        return n;
    }

    std::shared_ptr<YamlNode> ParseMap(size_t& i, int indent) {
        auto n = std::make_shared<YamlNode>();
        n->kind = YamlNode::Kind::Mapping;
        n->line = L[i].lineno;
        while (i < L.size() && L[i].indent == indent && !IsSeqItem(L[i].text)) {
            const std::string t = L[i].text;
            const int lineno = L[i].lineno;
            size_t c = FindKeySep(t);
            if (c == std::string::npos)
                throw YamlError("line " + std::to_string(lineno) + ": expected 'key: value'");
            std::string key = Unquote(t.substr(0, c), lineno);
            for (auto& kv : n->map)
                if (kv.first == key) throw YamlError("line " + std::to_string(lineno) + ": duplicate key '" + key + "'");
            std::string val = Trim(t.substr(c + 1));
            i++;
            if (!val.empty()) {
                n->map.emplace_back(key, ParseFlowOrScalar(val, lineno));
            } else if (i < L.size() && L[i].indent > indent) {
                n->map.emplace_back(key, ParseBlock(i, L[i].indent));
            } else if (i < L.size() && L[i].indent == indent && IsSeqItem(L[i].text)) {
                n->map.emplace_back(key, ParseSeq(i, indent));  // "key:\n- item" at the same column
            } else {
                n->map.emplace_back(key, std::make_shared<YamlNode>());
            }
        }
        return n;
    }
};

}  // namespace

const YamlNode& YamlNode::operator[](const std::string& key) const {
    if (kind == Kind::Mapping)
        for (auto& kv : map)
            if (kv.first == key) return *kv.second;
    return NullNode();
}

const YamlNode& YamlNode::operator[](size_t i) const {
    if (kind == Kind::Sequence && i < seq.size()) return *seq[i];
    return NullNode();
}

bool YamlNode::Has(const std::string& key) const {
    if (kind != Kind::Mapping) return false;
    for (auto& kv : map)
        if (kv.first == key) return !kv.second->IsNull();
    return false;
}

std::string YamlNode::AsString() const {
    if (kind != Kind::Scalar) throw YamlError("line " + std::to_string(line) + ": expected a scalar");
    return scalar;
}

double YamlNode::AsDouble() const {
    std::string s = AsString();
    errno = 0;
    char* end = nullptr;
    double v = std::strtod(s.c_str(), &end);
    if (end == s.c_str() || *end != '\0' || errno == ERANGE)
        throw YamlError("line " + std::to_string(line) + ": '" + s + "' is not a number");
    return v;
}

int YamlNode::AsInt() const {
    std::string s = AsString();
    errno = 0;
    char* end = nullptr;
    long v = std::strtol(s.c_str(), &end, 10);
    if (end == s.c_str() || *end != '\0' || errno == ERANGE || v < -2147483647L - 1 || v > 2147483647L)
        throw YamlError("line " + std::to_string(line) + ": '" + s + "' is not an integer");
    return (int)v;
}

bool YamlNode::AsBool() const {
    std::string s = AsString();
    if (s == "true" || s == "True" || s == "TRUE" || s == "yes" || s == "on") return true;
    if (s == "false" || s == "False" || s == "FALSE" || s == "no" || s == "off") return false;
    throw YamlError("line " + std::to_string(line) + ": '" + s + "' is not a boolean");
}

std::shared_ptr<YamlNode> YamlParse(const std::string& text) {
    std::vector<Line> lines;
    std::istringstream in(text);
    std::string raw;
    int lineno = 0;
    while (std::getline(in, raw)) {
        lineno++;
        if (!raw.empty() && raw.back() == '\r') raw.pop_back();
        for (char c : raw)
            if (c == '\t') {
                // YAML forbids tabs for indentation; only check the leading part.
                break;
            } else if (c != ' ') {
                break;
            }
        std::string s = StripComment(raw);
        std::string t = Trim(s);
        if (t.empty()) continue;
        if (t == "---" || t == "...") continue;
        int indent = 0;
        while (indent < (int)s.size() && s[indent] == ' ') indent++;
        if (indent < (int)s.size() && s[indent] == '\t')
            throw YamlError("line " + std::to_string(lineno) + ": tab used for indentation");
        lines.push_back({indent, t, lineno});
    }
    Parser p(std::move(lines));
    return p.ParseDocument();
}

std::shared_ptr<YamlNode> YamlLoadFile(const std::string& path) {
    std::ifstream f(path, std::ios::binary);
    if (!f) throw std::ios_base::failure("cannot open " + path);
    std::stringstream ss;
    ss << f.rdbuf();
    return YamlParse(ss.str());
}

}  // namespace ngi
