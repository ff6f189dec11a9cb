// POSIX-backed stand-in for the two Boost.Filesystem calls chiML makes
// (test infrastructure only).
#pragma once

#include <cerrno>
#include <cstdio>
#include <string>
#include <sys/stat.h>
#include <sys/types.h>

namespace boost {
namespace filesystem {

class path {
public:
    path() {}
    path(const char* s) : p_(s) {}
    path(const std::string& s) : p_(s) {}
    path& remove_filename() {
        std::size_t slash = p_.find_last_of('/');
        p_ = (slash == std::string::npos) ? std::string() : p_.substr(0, slash);
        return *this;
    }
    const std::string& string() const { return p_; }

private:
    std::string p_;
};

inline bool create_directories(const path& p) {
    const std::string& s = p.string();
    if (s.empty()) return false;
    bool made = false;
    for (std::size_t i = 1; i <= s.size(); ++i) {
        if (i == s.size() || s[i] == '/') {
            std::string part = s.substr(0, i);
            if (::mkdir(part.c_str(), 0755) == 0) made = true;
        }
    }
    return made;
}
inline bool remove(const path& p) { return std::remove(p.string().c_str()) == 0; }

}  // namespace filesystem
}  // namespace boost
