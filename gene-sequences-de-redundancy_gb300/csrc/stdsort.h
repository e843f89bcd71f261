// stdsort.h -- std::sort's exact permutation, computed on several host threads.
//
// readFile sorts the reads with std::sort (cuda-version/func.cu:111-113), and
// the order of equal-length reads decides which read becomes a
// representative, so the permutation must be std::sort's, ties included.
// libstdc++'s std::sort is an introsort: a loop that partitions the range
// around a median-of-three pivot, handles the right part recursively and
// continues with the left part, falls back to heapsort below a depth limit
// and leaves blocks of at most 16 elements; one insertion sort over the whole
// range then finishes those blocks.  Every part a partition produces is
// disjoint from the others and is processed from its own contents only, so
// running the loop's top levels here and the loops of the parts on threads
// performs the same element moves as the serial call.  The pieces are the
// library's own (the functions std::sort itself calls, same arguments), so
// the result is the library's permutation; with another standard library the
// call is plain std::sort.
#pragma once
#include <algorithm>
#include <iterator>
#include <thread>
#include <vector>

namespace gsdr {

#if defined(__GLIBCXX__)
// The introsort loop on [a, b) with `k` threads: while k > 1, one partition
// step of the loop (std::__introsort_loop), the right part to a new thread
// with half of them, the left part here with the rest.
template <class It, class Depth, class C>
void introsort_threads(It a, It b, Depth depth, C c, int k) {
    if (k <= 1 || b - a <= 16 || depth == 0) {
        std::__introsort_loop(a, b, depth, c);
        return;
    }
    --depth;
    It cut = std::__unguarded_partition_pivot(a, b, c);
    const int kr = k / 2;
    std::thread right([=]() { introsort_threads(cut, b, depth, c, kr); });
    introsort_threads(a, cut, depth, c, k - kr);
    right.join();
}
#endif

template <class It, class Comp>
void std_sort_threaded(It first, It last, Comp comp, int threads) {
#if defined(__GLIBCXX__)
    using Diff = typename std::iterator_traits<It>::difference_type;
    const Diff n = last - first;
    if (threads <= 1 || n < ((Diff)1 << 16)) {
        std::sort(first, last, comp);
        return;
    }
    // std::sort = std::__sort: the introsort loop with depth limit
    // 2 * floor(log2 n), then the final insertion sort
    auto c = __gnu_cxx::__ops::__iter_comp_iter(comp);
    introsort_threads(first, last, std::__lg(n) * 2, c, threads);
    std::__final_insertion_sort(first, last, c);
#else
    (void)threads;
    std::sort(first, last, comp);
#endif
}

// Threads for the host sort: the machine's cores, at most 16.
inline int sort_threads() {
    const unsigned h = std::thread::hardware_concurrency();
    return h == 0 ? 1 : (int)std::min(h, 16u);
}

}  // namespace gsdr
