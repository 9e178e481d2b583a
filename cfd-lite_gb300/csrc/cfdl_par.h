// cfdl_par.h -- host-side parallel loops and sorts for mesh preparation.
//
// Mesh set-up and case preparation are loops over cells and faces whose
// iterations write disjoint outputs, plus sorts under strict total orders;
// both give the same result on any number of threads.  The thread count is
// the hardware's, capped by a per-thread budget (host_threads()) that the
// serving loop lowers on its preparation threads so that they share the cores.
#pragma once
#include <algorithm>
#include <memory>
#include <new>
#include <thread>
#include <type_traits>
#include <utility>
#include <vector>

namespace cfdl {

// An allocator that leaves elements default-initialised (no zero-fill) when a
// vector is sized: a large table is then first touched, and its pages
// faulted in, by the parallel loop that fills every element, instead of by a
// serial fill that the loop overwrites.
template <class T> struct NoInitAlloc : std::allocator<T> {
    template <class U> struct rebind { using other = NoInitAlloc<U>; };
    NoInitAlloc() = default;
    template <class U> NoInitAlloc(const NoInitAlloc<U> &) noexcept {}
    template <class U> void construct(U *p) noexcept(std::is_nothrow_default_constructible<U>::value) {
        ::new (static_cast<void *>(p)) U;
    }
    template <class U, class... A> void construct(U *p, A &&...a) {
        ::new (static_cast<void *>(p)) U(std::forward<A>(a)...);
    }
};
template <class T> using FillVec = std::vector<T, NoInitAlloc<T>>;

// threads a parallel loop on this thread may use (0: all hardware threads)
inline int &host_threads() {
    static thread_local int n = 0;
    return n;
}

inline int par_threads(long n, long grain) {
    int hw = (int)std::max(1u, std::thread::hardware_concurrency());
    if (host_threads() > 0) hw = std::min(hw, host_threads());
    const long by_work = (n + grain - 1) / grain;
    return (int)std::max(1L, std::min<long>(std::min(hw, 32), by_work));
}

// f(begin, end) over [0, n) in contiguous chunks
template <class F> void parallel_for(long n, F f, long grain = 16384) {
    const int nt = par_threads(n, grain);
    if (nt <= 1) { if (n > 0) f(0L, n); return; }
    std::vector<std::thread> pool;
    const long chunk = (n + nt - 1) / nt;
    for (int t = 1; t < nt; t++) {
        const long b = t * chunk, e = std::min(n, b + chunk);
        if (b < e) pool.emplace_back([=] { f(b, e); });
    }
    f(0L, std::min(n, chunk));
    for (auto &th : pool) th.join();
}

// sort under a strict total order: chunks sorted in parallel, then merged
// pairwise in parallel rounds
template <class T, class Cmp> void parallel_sort(std::vector<T> &v, Cmp cmp) {
    const long n = (long)v.size();
    const int nt = par_threads(n, 1L << 16);
    if (nt <= 1) { std::sort(v.begin(), v.end(), cmp); return; }
    std::vector<long> cut(nt + 1);
    for (int t = 0; t <= nt; t++) cut[t] = n * t / nt;
    {
        std::vector<std::thread> pool;
        for (int t = 0; t < nt; t++)
            pool.emplace_back([&, t] { std::sort(v.begin() + cut[t], v.begin() + cut[t + 1], cmp); });
        for (auto &th : pool) th.join();
    }
    for (int width = 1; width < nt; width *= 2) {
        std::vector<std::thread> pool;
        for (int t = 0; t + width < nt; t += 2 * width) {
            const long b = cut[t], m = cut[t + width], e = cut[std::min(nt, t + 2 * width)];
            pool.emplace_back([&, b, m, e] { std::inplace_merge(v.begin() + b, v.begin() + m, v.begin() + e, cmp); });
        }
        for (auto &th : pool) th.join();
    }
}

}  // namespace cfdl
