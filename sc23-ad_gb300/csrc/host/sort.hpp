// utils::QuickSort (Library/utils/sort.hpp:31-51) restated: Hoare partition
// around the middle key, companion arrays permuted alongside.  The coarsening
// and the Matrix Market reader resolve ties through the exact sequence of
// swaps, so the same partition scheme is used wherever results depend on it.
#pragma once
#include <utility>

namespace sagb {

template <typename K, typename... Cs>
void hoare_sort(int lo, int hi, bool asc, K *key, Cs *...comps) {
    int l = lo, r = hi;
    const K piv = key[(lo + hi) / 2];
    for (;;) {
        if (asc) {
            while (key[l] < piv) l++;
            while (piv < key[r]) r--;
        } else {
            while (key[l] > piv) l++;
            while (piv > key[r]) r--;
        }
        if (l >= r) break;
        std::swap(key[l], key[r]);
        (std::swap(comps[l], comps[r]), ...);
        l++;
        r--;
    }
    if (lo < l - 1) hoare_sort(lo, l - 1, asc, key, comps...);
    if (r + 1 < hi) hoare_sort(r + 1, hi, asc, key, comps...);
}

}  // namespace sagb
