// JSON input tree for the chiML input file.
//
// The chiML reader (INPUTS/parallelInputs.cpp) looks values up through a
// Boost property tree, so the lookup rules here keep that behaviour: every
// scalar is held as text and converted on request by stream extraction (bools
// also accept true/false), dotted paths walk keyed children, arrays are
// children with empty keys, a missing path or failed conversion throws, and the
// defaulted form returns the default in either case. Comments introduced by
// "//" are removed line by line before parsing, as stripComments
// (parallelInputs.cpp:1625-1649) does.
#pragma once

#include <array>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace chiml {

struct InputError : public std::runtime_error {
    explicit InputError(const std::string& w) : std::runtime_error(w) {}
};

class JNode {
public:
    std::string text;
    std::vector<std::pair<std::string, JNode>> kids;

    const JNode* find(const std::string& path) const;
    const JNode& child(const std::string& path) const;
    bool has(const std::string& path) const { return find(path) != nullptr; }
    std::size_t size() const { return kids.size(); }

    template <typename T>
    static bool convert(const std::string& s, T& out) {
        std::istringstream iss(s);
        iss >> out;
        if (!iss.eof()) iss >> std::ws;
        return !(iss.fail() || iss.bad() || iss.get() != std::char_traits<char>::eof());
    }

    template <typename T>
    T value() const {
        T v{};
        if (!convert(text, v)) throw InputError("cannot convert value '" + text + "'");
        return v;
    }
    template <typename T>
    T get(const std::string& path) const {
        const JNode* n = find(path);
        if (!n) throw InputError("missing input key '" + path + "'");
        T v{};
        if (!convert(n->text, v)) throw InputError("cannot convert '" + path + "' = '" + n->text + "'");
        return v;
    }
    template <typename T>
    T get(const std::string& path, const T& def) const {
        const JNode* n = find(path);
        if (!n) return def;
        T v{};
        if (!convert(n->text, v)) return def;
        return v;
    }
    std::string gets(const std::string& path, const std::string& def) const { return get<std::string>(path, def); }
};

template <>
bool JNode::convert<bool>(const std::string& s, bool& out);
template <>
bool JNode::convert<std::string>(const std::string& s, std::string& out);

// Parses a file after removing "//" comments; throws InputError on bad JSON.
JNode parse_json_file(const std::string& path);
JNode parse_json_text(const std::string& text);

// Array helpers with the fallbacks of as_vector / as_ptArr (parallelInputs.hpp:333-430).
std::vector<double> as_vector(const JNode& n, const std::string& key);
std::vector<double> as_vector(const JNode& n, const std::string& key, double def, int sz);
std::array<double, 3> as_arr3(const JNode& n, const std::string& key, double def = 0.0);

}  // namespace chiml
