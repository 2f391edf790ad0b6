// std::sort's exact result, with the top of its recursion on several host threads.
//
// The pore stage must order the maximum balls exactly as the reference's std::sort does
// (PoreAndThroatComputer.cpp:121-122): the order among equal radii decides seeds and pore ids,
// so a different (e.g. stable or radix) sort would not do. libstdc++'s std::sort is an
// introsort: partition steps while a range holds more than 16 elements (heap sort once the
// depth limit is spent), then one insertion sort over the whole array. After a partition step
// the two sides are sorted independently, and the final insertion sort never moves an element
// out of the range it was partitioned into (the element before a range never compares after
// the range's elements), so running the same steps of the same library routines on the two
// sides in parallel, and the final insertion sort per side, gives the same permutation.
// This relies on libstdc++ (the library the reference and this code are built with); other
// standard libraries fall back to a plain std::sort.
#pragma once

#include <algorithm>
#include <system_error>
#include <thread>

namespace pma {

#if defined(__GLIBCXX__)
namespace detail {

template <class It, class Comp>
void ordered_sort_rec(It first, It last, long depth, Comp comp, int levels) {
    const long threshold = 16;  // libstdc++ _S_threshold
    if (levels == 0 || last - first <= threshold) {
        std::__introsort_loop(first, last, depth, comp);
        std::__final_insertion_sort(first, last, comp);
        return;
    }
    if (depth == 0) {
        std::__partial_sort(first, last, last, comp);
        return;
    }
    --depth;
    It cut = std::__unguarded_partition_pivot(first, last, comp);
    std::thread right;
    try {
        right = std::thread([=] { ordered_sort_rec(cut, last, depth, comp, levels - 1); });
    } catch (const std::system_error&) {  // no thread to be had: the same steps, in line
        ordered_sort_rec(cut, last, depth, comp, 0);
    }
    ordered_sort_rec(first, cut, depth, comp, levels - 1);
    if (right.joinable()) right.join();
}

}  // namespace detail

// Same result as std::sort(first, last, less); 2^levels tasks at most.
template <class It, class Less>
void ordered_sort(It first, It last, Less less, int levels = 3) {
    if (first == last) return;
    auto comp = __gnu_cxx::__ops::__iter_comp_iter(less);
    detail::ordered_sort_rec(first, last, static_cast<long>(std::__lg(last - first)) * 2, comp, levels);
}
#else
template <class It, class Less>
void ordered_sort(It first, It last, Less less, int = 3) {
    std::sort(first, last, less);
}
#endif

}  // namespace pma
