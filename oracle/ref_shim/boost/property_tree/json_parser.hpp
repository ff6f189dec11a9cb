// JSON reader for the ptree stand-in (test infrastructure only).
//
// Mirrors the published Boost.PropertyTree JSON mapping: objects become keyed
// children, arrays become children with empty keys, scalars are stored as
// their literal text (true/false/null included), strings are unescaped.
#pragma once

#include <boost/property_tree/ptree.hpp>

#include <cctype>
#include <fstream>
#include <sstream>
#include <string>

namespace boost {
namespace property_tree {
namespace json_parser {

struct json_parser_error : public ptree_error {
    explicit json_parser_error(const std::string& w) : ptree_error("json: " + w) {}
};

namespace detail {
class Reader {
public:
    explicit Reader(const std::string& s) : s_(s), i_(0) {}
    void parse(ptree& out) {
        ws();
        value(out);
        ws();
        if (i_ != s_.size()) fail("trailing characters");
    }

private:
    const std::string& s_;
    std::size_t i_;
    [[noreturn]] void fail(const char* why) {
        throw json_parser_error(std::string(why) + " at offset " + std::to_string(i_));
    }
    void ws() {
        while (i_ < s_.size() && std::isspace(static_cast<unsigned char>(s_[i_]))) ++i_;
    }
    char peek() { return i_ < s_.size() ? s_[i_] : '\0'; }
    void expect(char c) {
        if (peek() != c) fail("unexpected character");
        ++i_;
    }
    std::string str() {
        expect('"');
        std::string r;
        while (true) {
            if (i_ >= s_.size()) fail("unterminated string");
            char c = s_[i_++];
            if (c == '"') break;
            if (c == '\\') {
                char e = s_[i_++];
                switch (e) {
                    case 'n': r += '\n'; break;
                    case 't': r += '\t'; break;
                    case 'r': r += '\r'; break;
                    case 'b': r += '\b'; break;
                    case 'f': r += '\f'; break;
                    case 'u': {
                        unsigned v = std::stoul(s_.substr(i_, 4), nullptr, 16);
                        i_ += 4;
                        if (v < 0x80) r += static_cast<char>(v);
                        else if (v < 0x800) { r += static_cast<char>(0xC0 | (v >> 6)); r += static_cast<char>(0x80 | (v & 0x3F)); }
                        else { r += static_cast<char>(0xE0 | (v >> 12)); r += static_cast<char>(0x80 | ((v >> 6) & 0x3F)); r += static_cast<char>(0x80 | (v & 0x3F)); }
                        break;
                    }
                    default: r += e;
                }
            } else {
                r += c;
            }
        }
        return r;
    }
    void value(ptree& out) {
        ws();
        char c = peek();
        if (c == '{') {
            ++i_;
            ws();
            if (peek() == '}') { ++i_; return; }
            while (true) {
                ws();
                std::string k = str();
                ws();
                expect(':');
                ptree child;
                value(child);
                out.push_back(ptree::value_type(k, child));
                ws();
                if (peek() == ',') { ++i_; continue; }
                expect('}');
                return;
            }
        } else if (c == '[') {
            ++i_;
            ws();
            if (peek() == ']') { ++i_; return; }
            while (true) {
                ptree child;
                value(child);
                out.push_back(ptree::value_type("", child));
                ws();
                if (peek() == ',') { ++i_; continue; }
                expect(']');
                return;
            }
        } else if (c == '"') {
            out.data() = str();
        } else {
            std::size_t b = i_;
            while (i_ < s_.size() && (std::isalnum(static_cast<unsigned char>(s_[i_])) || s_[i_] == '-' || s_[i_] == '+' || s_[i_] == '.'))
                ++i_;
            if (b == i_) fail("bad value");
            out.data() = s_.substr(b, i_ - b);
        }
    }
};
}  // namespace detail

inline void read_json(const std::string& filename, ptree& pt) {
    std::ifstream in(filename);
    if (!in) throw json_parser_error("cannot open file " + filename);
    std::stringstream ss;
    ss << in.rdbuf();
    std::string text = ss.str();
    ptree tmp;
    detail::Reader(text).parse(tmp);
    pt = tmp;
}

}  // namespace json_parser
}  // namespace property_tree
}  // namespace boost
