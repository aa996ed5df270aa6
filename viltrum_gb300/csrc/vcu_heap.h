/*
 * vcu_heap.h -- the max-heap of (error, payload) pairs that drives adaptive refinement.
 *
 * viltrum keeps its regions in a std::vector ordered with std::push_heap / std::pop_heap by
 * "a.error < b.error" (src/nested/regions-generator-adaptive-heap.h:25-43), so WHICH region is
 * split among equal errors, and the order the regions are finally integrated in, are those of
 * libstdc++'s heap algorithms (GCC 13, bits/stl_heap.h).  This file restates that published
 * algorithm on two parallel arrays (keys and payloads) so the device makes the same choices:
 *   push: sift the new last element up while its parent compares less;
 *   pop:  move the last element out, move the root to the last slot, walk the hole from the
 *         root to a leaf always taking the larger child (the right one unless it is less than
 *         the left), fill a lone left child at the end for even lengths, then sift the saved
 *         element up from the hole.
 * Host and device compile the same code; tests/test_heap.py checks it against std::.
 */
#pragma once

#if defined(__CUDACC__)
#define VCU_HEAP_HD __host__ __device__ __forceinline__
#else
#define VCU_HEAP_HD inline
#endif

namespace vcu {

template <class K, class P>
VCU_HEAP_HD void heap_sift_up(K* key, P* pay, int hole, int top, K vk, P vp) {
    int parent = (hole - 1) / 2;
    while (hole > top && key[parent] < vk) {
        key[hole] = key[parent];
        pay[hole] = pay[parent];
        hole = parent;
        parent = (hole - 1) / 2;
    }
    key[hole] = vk;
    pay[hole] = vp;
}

/* the element at index len-1 has just been appended; restore the heap over [0, len) */
template <class K, class P> VCU_HEAP_HD void heap_push(K* key, P* pay, int len) {
    heap_sift_up(key, pay, len - 1, 0, key[len - 1], pay[len - 1]);
}

/* move the maximum to index len-1 and restore the heap over [0, len-1) */
template <class K, class P> VCU_HEAP_HD void heap_pop(K* key, P* pay, int len) {
    if (len <= 1) return;
    const int n = len - 1;
    const K vk = key[n];
    const P vp = pay[n];
    key[n] = key[0];
    pay[n] = pay[0];
    int hole = 0, child = 0;
    while (child < (n - 1) / 2) {
        child = 2 * (child + 1);
        if (key[child] < key[child - 1]) child--;
        key[hole] = key[child];
        pay[hole] = pay[child];
        hole = child;
    }
    if ((n & 1) == 0 && child == (n - 2) / 2) {
        child = 2 * (child + 1);
        key[hole] = key[child - 1];
        pay[hole] = pay[child - 1];
        hole = child - 1;
    }
    heap_sift_up(key, pay, hole, 0, vk, vp);
}

}  // namespace vcu
