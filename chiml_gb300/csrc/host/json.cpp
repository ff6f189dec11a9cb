#include "json.hpp"

#include <cctype>
#include <fstream>

namespace chiml {

template <>
bool JNode::convert<bool>(const std::string& s, bool& out) {
    {
        std::istringstream iss(s);
        iss >> out;
        if (!iss.fail()) {
            if (!iss.eof()) iss >> std::ws;
            if (!(iss.bad() || iss.get() != std::char_traits<char>::eof())) return true;
        }
    }
    std::istringstream iss(s);
    iss.setf(std::ios_base::boolalpha);
    iss >> out;
    if (!iss.eof()) iss >> std::ws;
    return !(iss.fail() || iss.bad() || iss.get() != std::char_traits<char>::eof());
}

template <>
bool JNode::convert<std::string>(const std::string& s, std::string& out) {
    out = s;
    return true;
}

const JNode* JNode::find(const std::string& path) const {
    const JNode* cur = this;
    std::size_t pos = 0;
    while (true) {
        std::size_t dot = path.find('.', pos);
        std::string key = path.substr(pos, dot == std::string::npos ? std::string::npos : dot - pos);
        const JNode* next = nullptr;
        for (auto& kv : cur->kids)
            if (kv.first == key) {
                next = &kv.second;
                break;
            }
        if (!next) return nullptr;
        cur = next;
        if (dot == std::string::npos) return cur;
        pos = dot + 1;
    }
}

const JNode& JNode::child(const std::string& path) const {
    const JNode* n = find(path);
    if (!n) throw InputError("missing input key '" + path + "'");
    return *n;
}

namespace {
class Parser {
public:
    explicit Parser(const std::string& s) : s_(s) {}
    JNode run() {
        JNode root;
        ws();
        value(root);
        ws();
        if (i_ != s_.size()) fail("trailing characters");
        return root;
    }

private:
    const std::string& s_;
    std::size_t i_ = 0;
    [[noreturn]] void fail(const char* why) {
        throw InputError(std::string("malformed JSON: ") + why + " at offset " + std::to_string(i_));
    }
    void ws() {
        while (i_ < s_.size() && std::isspace(static_cast<unsigned char>(s_[i_]))) ++i_;
    }
    char peek() const { return i_ < s_.size() ? s_[i_] : '\0'; }
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
            if (c == '"') return r;
            if (c != '\\') {
                r += c;
                continue;
            }
            if (i_ >= s_.size()) fail("bad escape");
            char e = s_[i_++];
            switch (e) {
                case 'n': r += '\n'; break;
                case 't': r += '\t'; break;
                case 'r': r += '\r'; break;
                case 'b': r += '\b'; break;
                case 'f': r += '\f'; break;
                case 'u': {
                    if (i_ + 4 > s_.size()) fail("bad unicode escape");
                    unsigned v = static_cast<unsigned>(std::stoul(s_.substr(i_, 4), nullptr, 16));
                    i_ += 4;
                    if (v < 0x80) {
                        r += static_cast<char>(v);
                    } else if (v < 0x800) {
                        r += static_cast<char>(0xC0 | (v >> 6));
                        r += static_cast<char>(0x80 | (v & 0x3F));
                    } else {
                        r += static_cast<char>(0xE0 | (v >> 12));
                        r += static_cast<char>(0x80 | ((v >> 6) & 0x3F));
                        r += static_cast<char>(0x80 | (v & 0x3F));
                    }
                    break;
                }
                default: r += e;
            }
        }
    }
    void value(JNode& out) {
        ws();
        char c = peek();
        if (c == '{') {
            ++i_;
            ws();
            if (peek() == '}') {
                ++i_;
                return;
            }
            while (true) {
                ws();
                std::string k = str();
                ws();
                expect(':');
                JNode child;
                value(child);
                out.kids.emplace_back(std::move(k), std::move(child));
                ws();
                if (peek() == ',') {
                    ++i_;
                    continue;
                }
                expect('}');
                return;
            }
        } else if (c == '[') {
            ++i_;
            ws();
            if (peek() == ']') {
                ++i_;
                return;
            }
            while (true) {
                JNode child;
                value(child);
                out.kids.emplace_back(std::string(), std::move(child));
                ws();
                if (peek() == ',') {
                    ++i_;
                    continue;
                }
                expect(']');
                return;
            }
        } else if (c == '"') {
            out.text = str();
        } else {
            std::size_t b = i_;
            while (i_ < s_.size() && (std::isalnum(static_cast<unsigned char>(s_[i_])) || s_[i_] == '-' ||
                                      s_[i_] == '+' || s_[i_] == '.'))
                ++i_;
            if (b == i_) fail("bad value");
            out.text = s_.substr(b, i_ - b);
        }
    }
};

// Removes everything from the first "//" of a line when the first '/' on the
// line is immediately followed by another (the rule of stripComments).
std::string strip_comments(const std::string& text) {
    std::string out;
    std::istringstream in(text);
    std::string line;
    while (std::getline(in, line)) {
        std::size_t f = line.find('/');
        if (f != std::string::npos && f + 1 < line.size() && line[f + 1] == '/') line.erase(f);
        out += line;
        out += '\n';
    }
    return out;
}
}  // namespace

JNode parse_json_text(const std::string& text) {
    std::string clean = strip_comments(text);
    return Parser(clean).run();
}

JNode parse_json_file(const std::string& path) {
    std::ifstream in(path);
    if (!in) throw InputError("cannot open input file '" + path + "'");
    std::stringstream ss;
    ss << in.rdbuf();
    return parse_json_text(ss.str());
}

std::vector<double> as_vector(const JNode& n, const std::string& key) {
    std::vector<double> r;
    for (auto& kv : n.child(key).kids) r.push_back(kv.second.value<double>());
    return r;
}

std::vector<double> as_vector(const JNode& n, const std::string& key, double def, int sz) {
    try {
        return as_vector(n, key);
    } catch (const InputError&) {
        return std::vector<double>(static_cast<std::size_t>(sz), def);
    }
}

std::array<double, 3> as_arr3(const JNode& n, const std::string& key, double def) {
    std::array<double, 3> r = {0.0, 0.0, 0.0};
    const JNode* c = n.find(key);
    if (!c) return {def, def, def};
    std::size_t i = 0;
    for (auto& kv : c->kids) {
        double v;
        if (!JNode::convert(kv.second.text, v)) return {def, def, def};
        if (i >= 3) throw InputError("array '" + key + "' has more than three entries");
        r[i++] = v;
    }
    return r;
}

}  // namespace chiml
