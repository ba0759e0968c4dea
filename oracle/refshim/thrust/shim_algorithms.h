// CPU launch shim: the two thrust algorithms the reference calls
// (core/neighborSearch.cu:3-17), on host memory.
//   sort_by_key:     stable sort of (key, value) by key.  thrust sorts int keys
//                    with a radix sort, which is stable, so std::stable_sort
//                    gives the same permutation.
//   inclusive_scan:  running sum.
#pragma once
#include <algorithm>
#include <cstddef>
#include <numeric>
#include <vector>

namespace thrust {

template <class T>
struct device_ptr {
    T* p;
    explicit device_ptr(T* q) : p(q) {}
};

template <class K, class V>
void sort_by_key(device_ptr<K> kb, device_ptr<K> ke, device_ptr<V> vb)
{
    const std::ptrdiff_t n = ke.p - kb.p;
    if (n <= 0) return;
    std::vector<std::ptrdiff_t> order(n);
    std::iota(order.begin(), order.end(), 0);
    std::stable_sort(order.begin(), order.end(),
                     [&](std::ptrdiff_t a, std::ptrdiff_t b) { return kb.p[a] < kb.p[b]; });
    std::vector<K> k2(n);
    std::vector<V> v2(n);
    for (std::ptrdiff_t i = 0; i < n; ++i) {
        k2[i] = kb.p[order[i]];
        v2[i] = vb.p[order[i]];
    }
    std::copy(k2.begin(), k2.end(), kb.p);
    std::copy(v2.begin(), v2.end(), vb.p);
}

template <class T>
void inclusive_scan(device_ptr<T> b, device_ptr<T> e, device_ptr<T> o)
{
    std::partial_sum(b.p, e.p, o.p);
}

}  // namespace thrust
