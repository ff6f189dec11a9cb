// Single-rank stand-in for the part of Boost.MPI that chiML's sources use.
//
// Test infrastructure only: it lets the unmodified reference sources be
// compiled into a one-process CPU binary whose outputs pin the oracle.
// Every collective degenerates to a copy; point-to-point messages are
// matched by tag through an in-process mailbox, so the self-sends the
// emitter code issues (parallelQE E/P exchange) complete as copies.
#pragma once

#include <algorithm>
#include <cstring>
#include <map>
#include <stdexcept>
#include <utility>
#include <vector>

namespace boost {
namespace mpi {

class environment {
public:
    environment() {}
    environment(int&, char**&) {}
};

namespace detail {
struct Pending {
    void* dst;
    std::size_t bytes;
};
// tag -> queue of payloads that arrived before their receive was posted
inline std::multimap<int, std::vector<char>>& mailbox() {
    static std::multimap<int, std::vector<char>> m;
    return m;
}
// tag -> receives posted before their send
inline std::multimap<int, Pending>& waiting() {
    static std::multimap<int, Pending> w;
    return w;
}
inline void deliver(int tag, const void* src, std::size_t bytes) {
    auto& w = waiting();
    auto it = w.find(tag);
    if (it != w.end()) {
        std::memcpy(it->second.dst, src, std::min(bytes, it->second.bytes));
        w.erase(it);
        return;
    }
    std::vector<char> payload(bytes);
    if (bytes) std::memcpy(payload.data(), src, bytes);
    mailbox().emplace(tag, std::move(payload));
}
inline void post_recv(int tag, void* dst, std::size_t bytes) {
    auto& m = mailbox();
    auto it = m.find(tag);
    if (it != m.end()) {
        std::memcpy(dst, it->second.data(), std::min(bytes, it->second.size()));
        m.erase(it);
        return;
    }
    waiting().emplace(tag, Pending{dst, bytes});
}
}  // namespace detail

struct status {
    int source() const { return 0; }
    int tag() const { return 0; }
};

class request {
public:
    status wait() { return status(); }
    bool test() { return true; }
    void cancel() {}
};

template <typename It>
void wait_all(It, It) {
    if (!detail::waiting().empty())
        throw std::logic_error("single-rank mpi stand-in: a receive has no matching send");
}

class communicator {
public:
    communicator() {}
    virtual ~communicator() {}
    int rank() const { return 0; }
    int size() const { return 1; }
    void barrier() const {}

    template <typename T>
    request isend(int, int tag, const T* p, int n) const {
        detail::deliver(tag, p, sizeof(T) * static_cast<std::size_t>(n));
        return request();
    }
    template <typename T>
    request irecv(int, int tag, T* p, int n) const {
        detail::post_recv(tag, p, sizeof(T) * static_cast<std::size_t>(n));
        return request();
    }
    template <typename T>
    request isend(int dest, int tag, const std::vector<T>& v) const {
        return isend(dest, tag, v.data(), static_cast<int>(v.size()));
    }
    template <typename T>
    void send(int, int tag, const std::vector<T>& v) const {
        std::size_t n = v.size();
        detail::deliver(tag + (1 << 28), &n, sizeof(n));
        detail::deliver(tag, v.data(), sizeof(T) * n);
    }
    template <typename T>
    void recv(int, int tag, std::vector<T>& v) const {
        std::size_t n = 0;
        detail::post_recv(tag + (1 << 28), &n, sizeof(n));
        v.resize(n);
        detail::post_recv(tag, v.data(), sizeof(T) * n);
    }
    template <typename T>
    void send(int, int tag, const T& v) const {
        detail::deliver(tag, &v, sizeof(T));
    }
    template <typename T>
    void recv(int, int tag, T& v) const {
        detail::post_recv(tag, &v, sizeof(T));
    }
};

template <typename T>
void broadcast(const communicator&, T&, int) {}
template <typename T>
void broadcast(const communicator&, T*, int, int) {}

template <typename T>
void gather(const communicator&, const T& in, std::vector<T>& out, int) {
    out.assign(1, in);
}
template <typename T>
void gather(const communicator&, const T&, int) {}

template <typename T>
void all_gather(const communicator&, const T& in, std::vector<T>& out) {
    out.assign(1, in);
}

}  // namespace mpi
}  // namespace boost
