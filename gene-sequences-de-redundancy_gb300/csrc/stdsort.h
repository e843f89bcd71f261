// stdsort.h -- std::sort's exact permutation, computed on several host threads.
//
// readFile sorts the reads with std::sort (cuda-version/func.cu:111-113), and
// the order of equal-length reads decides which read becomes a
// representative, so the permutation must be std::sort's, ties included.
// libstdc++'s std::sort is an introsort: a loop that moves the median of three
// to the front, partitions the rest around it (an unguarded Hoare partition),
// handles the right part recursively and continues with the left part, falls
// back to heapsort below a depth limit and leaves blocks of at most 16
// elements; one insertion sort over the whole range then finishes the blocks.
//
// Every part a partition produces is disjoint from the others and is
// processed from its own contents only, and the final insertion sort never
// moves an element across a partition boundary (an element right of a cut is
// never ordered before one left of it), so the parts can be sorted
// independently -- each to the end, insertion sort included -- with the same
// element moves as the serial call.  Here:
//   * parts of at least kTeamPart elements are partitioned by all threads
//     together (team_partition): the Hoare loop swaps the k-th element from
//     the left that is not before the pivot with the k-th element from the
//     right that is not after it, for as long as the first lies left of the
//     second (the scans read only positions no swap has touched until then,
//     so both sequences of positions come from the original range: per-thread
//     counts, a prefix sum, a binary search for the count K), and returns
//     where the scans meet: the (K+1)-th left position, or the K-th right
//     position if that comes first (it holds a swapped-in left element); the
//     swaps are independent;
//   * smaller parts go to a shared stack, from which the threads take parts,
//     split them with the library's own partition step while they are large,
//     and finish each piece with the library's introsort loop and insertion
//     sort.
// The pieces are the library's own (the functions std::sort calls), so the
// result is the library's permutation; with another standard library the call
// is plain std::sort.
#pragma once
#include <algorithm>
#include <atomic>
#include <cstdlib>
#include <functional>
#include <iterator>
#include <mutex>
#include <thread>
#include <vector>

namespace gsdr {

#if defined(__GLIBCXX__)
namespace sort_detail {

constexpr long kTeamPart = 1 << 16;  // parts partitioned by the whole team
constexpr long kSplitPart = 1 << 13;  // stack parts still split before the loop

class SpinBarrier {
  public:
    explicit SpinBarrier(int n) : n_(n) {}
    void wait() {
        const int g = gen_.load(std::memory_order_acquire);
        if (count_.fetch_add(1, std::memory_order_acq_rel) == n_ - 1) {
            count_.store(0, std::memory_order_relaxed);
            gen_.fetch_add(1, std::memory_order_release);
        } else {
            while (gen_.load(std::memory_order_acquire) == g) std::this_thread::yield();
        }
    }

  private:
    const int n_;
    std::atomic<int> count_{0};
    std::atomic<int> gen_{0};
};

template <class It, class Depth>
struct Part {
    It a, b;
    Depth depth;
};

// State shared by the team while it sorts one range.
template <class It, class Depth>
struct Team {
    explicit Team(int n) : threads(n), bar(n), cnt_l(n), cnt_r(n) {}
    const int threads;
    SpinBarrier bar;
    std::vector<long> cnt_l, cnt_r;  // stops per thread chunk
    std::vector<long> lpos, rpos;    // stop positions (offsets from the part's start)
    long cut = 0;
    bool serial = false;  // the crossing was not found: thread 0 partitioned serially
    // stack of parts for the second phase
    std::mutex mu;
    std::vector<Part<It, Depth>> stack;
    std::atomic<long> pending{0};  // parts pushed and not yet finished
};

// std::__unguarded_partition_pivot(a, b, c) by the whole team (thread t of
// T); every thread returns the same cut.
template <class It, class Depth, class C>
It team_partition(Team<It, Depth>& tm, int t, It a, It b, C c) {
    const int T = tm.threads;
    if (t == 0) {
        std::__move_median_to_first(a, a + 1, a + (b - a) / 2, b - 1, c);
        tm.lpos.resize((size_t)(b - a));
        tm.rpos.resize((size_t)(b - a));
    }
    tm.bar.wait();
    // the Hoare loop runs on [a + 1, b) with the pivot at a
    const long m = (long)(b - a) - 1;
    const long lo = 1 + m * t / T, hi = 1 + m * (t + 1) / T;
    long nl = 0, nr = 0;
    for (long i = lo; i < hi; i++) {
        nl += !c(a + i, a);  // left scan stops: not before the pivot
        nr += !c(a, a + i);  // right scan stops: not after the pivot
    }
    tm.cnt_l[t] = nl;
    tm.cnt_r[t] = nr;
    tm.bar.wait();
    long ol = 0, orr = 0;
    for (int s = 0; s < t; s++) ol += tm.cnt_l[s];
    for (int s = t + 1; s < T; s++) orr += tm.cnt_r[s];
    for (long i = lo; i < hi; i++)
        if (!c(a + i, a)) tm.lpos[ol++] = i;
    for (long i = hi - 1; i >= lo; i--)
        if (!c(a, a + i)) tm.rpos[orr++] = i;
    tm.bar.wait();
    if (t == 0) {
        long tl = 0, tr = 0;
        for (int s = 0; s < T; s++) {
            tl += tm.cnt_l[s];
            tr += tm.cnt_r[s];
        }
        // K = number of swaps: lpos[k] < rpos[k] holds for k < K (lpos rises,
        // rpos falls); the loop returns at the K-th left stop
        long lo_k = 0, hi_k = std::min(tl, tr);
        while (lo_k < hi_k) {
            const long mid = (lo_k + hi_k) / 2;
            if (tm.lpos[mid] < tm.rpos[mid]) lo_k = mid + 1;
            else hi_k = mid;
        }
        // after K swaps the left scan stops at the next left stop, or earlier
        // at the position of the K-th right stop (it now holds the K-th left
        // stop's element); either way it has met the right scan there
        tm.serial = lo_k == 0 && tl == 0;  // no left stop at all: not the library's case
        if (tm.serial) tm.cut = (long)(std::__unguarded_partition(a + 1, b, a, c) - a);
        else if (lo_k == 0) tm.cut = tm.lpos[0];
        else if (lo_k < tl && tm.lpos[lo_k] < tm.rpos[lo_k - 1]) tm.cut = tm.lpos[lo_k];
        else tm.cut = tm.rpos[lo_k - 1];
        tm.cnt_l[0] = lo_k;  // the swap count, for the next step
    }
    tm.bar.wait();
    if (!tm.serial) {
        const long K = tm.cnt_l[0];
        for (long k = K * t / T; k < K * (t + 1) / T; k++)
            std::iter_swap(a + tm.lpos[k], a + tm.rpos[k]);
    }
    It cut = a + tm.cut;
    tm.bar.wait();  // swaps done, and the shared state free for the next part
    return cut;
}

// The library's introsort loop on a part, then its insertion sort.
template <class It, class Depth, class C>
void finish_part(It a, It b, Depth depth, C c) {
    std::__introsort_loop(a, b, depth, c);
    if (b - a > 1) std::__insertion_sort(a, b, c);
}

// Thread t of the team: first the team partitions, then parts from the stack.
template <class It, class Depth, class C>
void team_sort(Team<It, Depth>& tm, int t, It first, It last, Depth depth0, C c) {
    using P = Part<It, Depth>;
    // phase 1: every thread walks the same list of parts and takes part in
    // each team partition, so all keep identical lists
    std::vector<P> cur{{first, last, depth0}}, small;
    while (!cur.empty()) {
        std::vector<P> next;
        for (const P& p : cur) {
            if (p.b - p.a < kTeamPart || p.depth == 0) {
                small.push_back(p);
                continue;
            }
            It cut = team_partition(tm, t, p.a, p.b, c);
            next.push_back({p.a, cut, p.depth - 1});
            next.push_back({cut, p.b, p.depth - 1});
        }
        cur.swap(next);
    }
    if (t == 0) {
        std::lock_guard<std::mutex> g(tm.mu);
        tm.stack = small;
        tm.pending.store((long)small.size(), std::memory_order_release);
    }
    tm.bar.wait();
    // phase 2: parts from the stack; a large part is split by the library's
    // partition step (the right piece back to the stack) before the loop
    while (tm.pending.load(std::memory_order_acquire) > 0) {
        P p{first, first, 0};
        bool got = false;
        {
            std::lock_guard<std::mutex> g(tm.mu);
            if (!tm.stack.empty()) {
                p = tm.stack.back();
                tm.stack.pop_back();
                got = true;
            }
        }
        if (!got) {  // others still split or finish parts
            std::this_thread::yield();
            continue;
        }
        while (p.b - p.a > kSplitPart && p.depth != 0) {
            --p.depth;
            It cut = std::__unguarded_partition_pivot(p.a, p.b, c);
            {
                std::lock_guard<std::mutex> g(tm.mu);
                tm.stack.push_back({cut, p.b, p.depth});
                tm.pending.fetch_add(1, std::memory_order_acq_rel);
            }
            p.b = cut;
        }
        finish_part(p.a, p.b, p.depth, c);
        tm.pending.fetch_sub(1, std::memory_order_acq_rel);
    }
}

}  // namespace sort_detail
#endif

// after(t, T), if given, runs on every thread t of the T that sorted, once the
// permutation is final (a parallel pass over the sorted range, e.g. a gather
// by the permutation, on threads that already exist).
template <class It, class Comp>
void std_sort_threaded(It first, It last, Comp comp, int threads,
                       const std::function<void(int, int)>& after = {}) {
#if defined(__GLIBCXX__)
    using Diff = typename std::iterator_traits<It>::difference_type;
    const Diff n = last - first;
    if (threads <= 1 || n < ((Diff)1 << 16)) {
        std::sort(first, last, comp);
        if (after) after(0, 1);
        return;
    }
    // std::sort = std::__sort: the introsort loop with depth limit
    // 2 * floor(log2 n), then the final insertion sort
    auto c = __gnu_cxx::__ops::__iter_comp_iter(comp);
    using Depth = decltype(std::__lg(n) * 2);
    sort_detail::Team<It, Depth> tm(threads);
    const Depth depth0 = std::__lg(n) * 2;
    // the workers start together once all exist (a barrier needs every one of
    // them); if a thread cannot be created, those that exist leave and the
    // call is a plain std::sort
    std::atomic<int> go{0};
    std::vector<std::thread> pool;
    try {
        for (int t = 1; t < threads; t++)
            pool.emplace_back([&, t]() {
                int g;
                while ((g = go.load(std::memory_order_acquire)) == 0) std::this_thread::yield();
                if (g > 0) {
                    sort_detail::team_sort(tm, t, first, last, depth0, c);
                    if (after) {
                        tm.bar.wait();  // every part finished
                        after(t, threads);
                    }
                }
            });
    } catch (...) {
        go.store(-1, std::memory_order_release);
        for (auto& th : pool) th.join();
        std::sort(first, last, comp);
        if (after) after(0, 1);
        return;
    }
    go.store(1, std::memory_order_release);
    sort_detail::team_sort(tm, 0, first, last, depth0, c);
    if (after) {
        tm.bar.wait();
        after(0, threads);
    }
    for (auto& th : pool) th.join();
#else
    (void)threads;
    std::sort(first, last, comp);
    if (after) after(0, 1);
#endif
}

// Threads for the host sort: the machine's cores, at most 16.
// Threads of the host sort: the hardware threads, at most 16; GSDR_SORT_THREADS
// overrides (1 = plain std::sort).
inline int sort_threads() {
    if (const char* e = std::getenv("GSDR_SORT_THREADS")) {
        const int v = std::atoi(e);
        if (v >= 1) return std::min(v, 64);
    }
    const unsigned h = std::thread::hardware_concurrency();
    return h == 0 ? 1 : (int)std::min(h, 16u);
}

}  // namespace gsdr
