//  vtkio.h -- host machinery of the drop-in VTK writers and readers (vtkexport.h,
//  vtkxmlexport.h, vtkimport.h, vtkxmlimport.h). Not on the GPU path.
//
//  Writers: the caller's functors are evaluated on the calling thread (the arrays they read may
//  change as soon as the call returns); the values are then formatted in parallel and written
//  by one background thread per file, in call order, so the solver goes on while a large field
//  is being written. A file is complete when its exporter is destroyed. The text is the
//  reference's std::ostream output byte for byte: default stream formatting prints a floating
//  value as printf's %g (6 significant digits) and an integer as an integer.
//
//  Readers: the file is read once into memory and scanned with the reference's token / line
//  rules; numbers are converted as std::istream does (strtod / strtof / strtoll).
#pragma once
#include <algorithm>
#include <condition_variable>
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <deque>
#include <fstream>
#include <functional>
#include <iterator>
#include <mutex>
#include <string>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

namespace PANSLBM2 {
namespace vtkio {

//  Set by the device runtime (gpu/runtime.h): brings the host arrays that saving collides left on
//  the device up to date before an exporter's functors read them. Unset for host-only use.
inline void (*&host_sync_hook())() {
    static void (*h)() = nullptr;
    return h;
}
inline void host_sync() {
    if (host_sync_hook()) host_sync_hook()();
}

//  one value as a default-formatted std::ostream prints it
struct Val {
    double d;
    long long i;
    bool isint;
};
template <class V>
inline Val val(V v) {
    if constexpr (std::is_integral<V>::value) return Val{0.0, (long long)v, true};
    else return Val{(double)v, 0, false};
}
inline void put(std::string &s, const Val &v) {
    char b[48];
    const int n = v.isint ? std::snprintf(b, sizeof b, "%lld", v.i) : std::snprintf(b, sizeof b, "%g", v.d);
    s.append(b, (size_t)n);
}
inline void put(std::string &s, double d) { put(s, Val{d, 0, false}); }
inline void put_int(std::string &s, long long i) { put(s, Val{0.0, i, true}); }

//  text of nodes [0, n): fn(out, node) appends one node's text; chunks run on several threads
template <class Fn>
std::string format_nodes(size_t n, Fn fn) {
    size_t nt = std::max(1u, std::min(16u, std::thread::hardware_concurrency()));
    if (n < (size_t)1 << 15) nt = 1;
    std::vector<std::string> part(nt);
    auto work = [&](size_t t) {
        const size_t lo = n * t / nt, hi = n * (t + 1) / nt;
        part[t].reserve((hi - lo) * 24);
        for (size_t node = lo; node < hi; ++node) fn(part[t], node);
    };
    std::vector<std::thread> th;
    for (size_t t = 1; t < nt; ++t) th.emplace_back(work, t);
    work(0);
    for (auto &x : th) x.join();
    size_t total = 0;
    for (auto &p : part) total += p.size();
    std::string out;
    out.reserve(total);
    for (auto &p : part) out += p;
    return out;
}

//  A file written by one background thread: tasks run in the order they were posted, each with
//  the file handle (the writers keep their seekp / tellp bookkeeping inside the tasks, on that
//  thread).
class AsyncFile {
public:
    explicit AsyncFile(const std::string &path) : fp_(std::fopen(path.c_str(), "wb")), worker_([this] { run(); }) {}
    AsyncFile(const AsyncFile &) = delete;
    ~AsyncFile() {
        {
            std::lock_guard<std::mutex> lk(mu_);
            done_ = true;
        }
        cv_.notify_one();
        worker_.join();
        if (fp_) std::fclose(fp_);
    }
    void post(std::function<void(std::FILE *)> task) {
        {
            std::lock_guard<std::mutex> lk(mu_);
            tasks_.push_back(std::move(task));
        }
        cv_.notify_one();
    }

private:
    void run() {
        for (;;) {
            std::function<void(std::FILE *)> t;
            {
                std::unique_lock<std::mutex> lk(mu_);
                cv_.wait(lk, [this] { return done_ || !tasks_.empty(); });
                if (tasks_.empty()) return;
                t = std::move(tasks_.front());
                tasks_.pop_front();
            }
            if (fp_) t(fp_);
        }
    }
    std::FILE *fp_;
    std::mutex mu_;
    std::condition_variable cv_;
    std::deque<std::function<void(std::FILE *)>> tasks_;
    bool done_ = false;
    std::thread worker_;
};
inline void write_at(std::FILE *fp, long long offset, const std::string &s) {
    std::fseek(fp, (long)offset, SEEK_SET);
    std::fwrite(s.data(), 1, s.size(), fp);
}

//  ---------------------------------------------------------------- readers
inline std::string slurp(const std::string &path) {
    std::ifstream in(path, std::ios::binary);
    if (!in) return std::string();
    return std::string(std::istreambuf_iterator<char>(in), std::istreambuf_iterator<char>());
}
inline bool is_space(char c) { return c == ' ' || c == '\t' || c == '\n' || c == '\r' || c == '\v' || c == '\f'; }

//  whitespace tokens of a text, read in order from a cursor (std::istream >> semantics)
struct Tokens {
    const std::string *text = nullptr;
    size_t pos = 0;
    bool next(const char *&p, size_t &len) {
        const std::string &s = *text;
        while (pos < s.size() && is_space(s[pos])) ++pos;
        if (pos >= s.size()) return false;
        const size_t b = pos;
        while (pos < s.size() && !is_space(s[pos])) ++pos;
        p = s.data() + b;
        len = pos - b;
        return true;
    }
    bool word(std::string &w) {
        const char *p;
        size_t len;
        if (!next(p, len)) return false;
        w.assign(p, len);
        return true;
    }
    template <class V>
    bool number(V &v) {
        const char *p;
        size_t len;
        if (!next(p, len)) return false;
        if constexpr (std::is_same<V, float>::value) v = std::strtof(p, nullptr);
        else if constexpr (std::is_same<V, long double>::value) v = std::strtold(p, nullptr);
        else if constexpr (std::is_floating_point<V>::value) v = (V)std::strtod(p, nullptr);
        else v = (V)std::strtoll(p, nullptr, 10);
        return true;
    }
};

//  std::getline over a text from a cursor
inline bool getline(const std::string &s, size_t &pos, std::string &line) {
    if (pos >= s.size()) return false;
    size_t e = s.find('\n', pos);
    if (e == std::string::npos) e = s.size();
    line.assign(s, pos, e - pos);
    pos = e < s.size() ? e + 1 : e;
    return true;
}

}  // namespace vtkio
}  // namespace PANSLBM2
