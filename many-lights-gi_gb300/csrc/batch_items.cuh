// Work-item walk of a persistent pass over the batch view table. Block b takes the pass's items
// b, b + gridDim.x, ... in increasing order, so the view an item belongs to only moves forward; the
// pass's running item counts are cached in shared memory (when they fit) and walked, not searched.
#pragma once

#include "kernels.h"

namespace mlgi {

constexpr int kBatchPrefixCache = 256;  // views whose running counts fit the shared-memory cache

struct ItemWalk {
    const int* p;  // running item counts of the pass: p[v] = first item of view v, p[n] = total
    int n, v;
    int total;

    // g_pre: the pass's counts in global memory; s_pre: kBatchPrefixCache + 1 ints of shared memory.
    // Called by every thread of the block.
    __device__ __forceinline__ void init(const int* g_pre, const int n_views, int* s_pre) {
        const bool cached = n_views <= kBatchPrefixCache;
        if (cached) {
            for (int i = threadIdx.x; i <= n_views; i += blockDim.x) s_pre[i] = __ldg(g_pre + i);
            __syncthreads();
        }
        p = cached ? s_pre : g_pre;
        n = n_views;
        v = 0;
        total = p[n_views];
    }
    // the view of `item` (items of one block must come in increasing order)
    __device__ __forceinline__ int view(const int item) {
        while (v + 1 < n && p[v + 1] <= item) ++v;
        return v;
    }
    // the item's index inside its view (after view(item))
    __device__ __forceinline__ int local(const int item) const { return item - p[v]; }
};

}  // namespace mlgi
