// Minimal stand-in for boost::property_tree::ptree as chiML's input reader uses it.
//
// Test infrastructure only (see ../mpi.hpp). Semantics follow the published
// Boost.PropertyTree behaviour that parallelInputs.cpp relies on: values are
// strings converted on demand with stream extraction (bools also accept
// true/false), dotted paths walk child keys, the first child with a key wins,
// a missing path throws ptree_bad_path, a failed conversion ptree_bad_data, and
// get<T>(path, default) returns the default in either case.
#pragma once

#include <iterator>
#include <sstream>
#include <stdexcept>
#include <string>
#include <utility>
#include <vector>

namespace boost {
namespace property_tree {

struct ptree_error : public std::runtime_error {
    explicit ptree_error(const std::string& w) : std::runtime_error(w) {}
};
struct ptree_bad_path : public ptree_error {
    explicit ptree_bad_path(const std::string& w) : ptree_error("No such node (" + w + ")") {}
};
struct ptree_bad_data : public ptree_error {
    explicit ptree_bad_data(const std::string& w) : ptree_error("conversion of data to type failed (" + w + ")") {}
};

namespace detail {
template <typename T>
inline bool convert(const std::string& s, T& out) {
    std::istringstream iss(s);
    iss >> out;
    if (!iss.eof()) iss >> std::ws;
    if (iss.fail() || iss.bad() || iss.get() != std::char_traits<char>::eof()) return false;
    return true;
}
template <>
inline bool convert<bool>(const std::string& s, bool& out) {
    std::istringstream iss(s);
    iss >> out;
    if (iss.fail()) {
        iss.clear();
        iss.str(s);
        iss.setf(std::ios_base::boolalpha);
        iss >> out;
    }
    if (!iss.eof()) iss >> std::ws;
    if (iss.fail() || iss.bad() || iss.get() != std::char_traits<char>::eof()) return false;
    return true;
}
template <>
inline bool convert<std::string>(const std::string& s, std::string& out) {
    out = s;
    return true;
}
}  // namespace detail

class ptree {
public:
    typedef std::string key_type;
    typedef std::string data_type;
    typedef std::pair<const std::string, ptree> value_type;
    typedef std::vector<value_type>::iterator iterator;
    typedef std::vector<value_type>::const_iterator const_iterator;

    ptree() {}
    explicit ptree(const std::string& d) : data_(d) {}
    ptree(const ptree& o) : data_(o.data_), kids_(o.kids_) {}
    ptree& operator=(const ptree& o) {
        if (this != &o) {
            data_ = o.data_;
            kids_.clear();
            for (auto& kv : o.kids_) kids_.emplace_back(kv.first, kv.second);
        }
        return *this;
    }

    iterator begin() { return kids_.begin(); }
    iterator end() { return kids_.end(); }
    const_iterator begin() const { return kids_.begin(); }
    const_iterator end() const { return kids_.end(); }
    std::size_t size() const { return kids_.size(); }
    bool empty() const { return kids_.empty(); }
    std::string& data() { return data_; }
    const std::string& data() const { return data_; }

    iterator push_back(const value_type& v) {
        kids_.emplace_back(v.first, v.second);
        return kids_.end() - 1;
    }
    iterator find_key(const std::string& k) {
        for (auto it = kids_.begin(); it != kids_.end(); ++it)
            if (it->first == k) return it;
        return kids_.end();
    }
    const_iterator find_key(const std::string& k) const {
        for (auto it = kids_.begin(); it != kids_.end(); ++it)
            if (it->first == k) return it;
        return kids_.end();
    }
    std::size_t count(const std::string& k) const {
        std::size_t n = 0;
        for (auto& kv : kids_) n += (kv.first == k);
        return n;
    }

    const ptree* walk(const std::string& path) const {
        const ptree* cur = this;
        std::size_t pos = 0;
        while (true) {
            std::size_t dot = path.find('.', pos);
            std::string key = path.substr(pos, dot == std::string::npos ? std::string::npos : dot - pos);
            auto it = cur->find_key(key);
            if (it == cur->kids_.end()) return nullptr;
            cur = &it->second;
            if (dot == std::string::npos) return cur;
            pos = dot + 1;
        }
    }

    ptree& get_child(const std::string& path) {
        const ptree* p = walk(path);
        if (!p) throw ptree_bad_path(path);
        return const_cast<ptree&>(*p);
    }
    const ptree& get_child(const std::string& path) const {
        const ptree* p = walk(path);
        if (!p) throw ptree_bad_path(path);
        return *p;
    }

    template <typename T>
    T get_value() const {
        T v{};
        if (!detail::convert<T>(data_, v)) throw ptree_bad_data(data_);
        return v;
    }
    template <typename T>
    T get(const std::string& path) const {
        return get_child(path).template get_value<T>();
    }
    template <typename T>
    T get(const std::string& path, const T& def) const {
        const ptree* p = walk(path);
        if (!p) return def;
        T v{};
        if (!detail::convert<T>(p->data_, v)) return def;
        return v;
    }
    std::string get(const std::string& path, const char* def) const {
        return get<std::string>(path, std::string(def));
    }

private:
    std::string data_;
    std::vector<value_type> kids_;
};

}  // namespace property_tree
}  // namespace boost
