// Stand-in for orlp/pdqsort (pinned by the reference at commit b1ef26a5, not present here).
// pdqsort is an unstable sort, so equal keys may come out in any order; this stand-in uses a
// stable sort so that the oracle's tie order is deterministic and can be reproduced exactly by
// this project's own CAPT builder.  For keys without ties both orders are identical.
#pragma once
#include <algorithm>

template <class It, class Cmp>
inline void pdqsort_branchless(It begin, It end, Cmp cmp)
{
    std::stable_sort(begin, end, cmp);
}

template <class It, class Cmp>
inline void pdqsort(It begin, It end, Cmp cmp)
{
    std::stable_sort(begin, end, cmp);
}
