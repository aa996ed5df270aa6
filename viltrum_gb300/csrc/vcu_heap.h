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
#include <cstddef>

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

/* The same two algorithms on packed (key, payload) entries, for heaps too large for shared
 * memory, through an accessor:
 *   HeapArray: element i at h[i];
 *   HeapSplit: elements below `cap` (odd) at top[i] (shared memory), the others at rest[i] (global).
 * In both, the two children of any element (2i+1, 2i+2) form one 16-byte aligned pair (h + 1,
 * top + 1 and rest + 1 are 16-byte aligned, and with an odd cap no pair straddles the two arrays),
 * which the device reads with a single load. */
struct HeapEntry {
    float key;
    int pay;
};

VCU_HEAP_HD void heap_load_pair(const HeapEntry* p, HeapEntry& l, HeapEntry& r) {
#if defined(__CUDA_ARCH__)
    const float4 pair = *reinterpret_cast<const float4*>(p);
    l = HeapEntry{pair.x, __float_as_int(pair.y)};
    r = HeapEntry{pair.z, __float_as_int(pair.w)};
#else
    l = p[0];
    r = p[1];
#endif
}

struct HeapArray {
    HeapEntry* h;
    VCU_HEAP_HD HeapEntry get(int i) const { return h[i]; }
    VCU_HEAP_HD void set(int i, HeapEntry e) const { h[i] = e; }
    VCU_HEAP_HD void pair(int left, HeapEntry& l, HeapEntry& r) const { heap_load_pair(h + left, l, r); }
};

struct HeapSplit {
    HeapEntry* top;
    HeapEntry* rest;
    int cap;
    VCU_HEAP_HD HeapEntry get(int i) const { return i < cap ? top[i] : rest[i]; }
    VCU_HEAP_HD void set(int i, HeapEntry e) const {
        if (i < cap) top[i] = e;
        else rest[i] = e;
    }
    VCU_HEAP_HD void pair(int left, HeapEntry& l, HeapEntry& r) const {
        heap_load_pair((left < cap ? top : rest) + left, l, r);
    }
};

template <class A> VCU_HEAP_HD void heap_sift_up_entries(const A& h, int hole, HeapEntry v) {
    int parent = (hole - 1) / 2;
    while (hole > 0) {
        const HeapEntry pe = h.get(parent);
        if (!(pe.key < v.key)) break;
        h.set(hole, pe);
        hole = parent;
        parent = (hole - 1) / 2;
    }
    h.set(hole, v);
}

template <class A> VCU_HEAP_HD void heap_push_entries(const A& h, int len) {
    heap_sift_up_entries(h, len - 1, h.get(len - 1));
}

template <class A> VCU_HEAP_HD void heap_pop_entries(const A& h, int len) {
    if (len <= 1) return;
    const int n = len - 1;
    const HeapEntry v = h.get(n);
    h.set(n, h.get(0));
    int hole = 0, child = 0;
    while (child < (n - 1) / 2) {
        child = 2 * (child + 1);
        HeapEntry left, right;
        h.pair(child - 1, left, right);
        const bool take_left = right.key < left.key;
        if (take_left) child--;
        h.set(hole, take_left ? left : right);
        hole = child;
    }
    if ((n & 1) == 0 && child == (n - 2) / 2) {
        child = 2 * (child + 1);
        h.set(hole, h.get(child - 1));
        hole = child - 1;
    }
    heap_sift_up_entries(h, hole, v);
}

/* The same two algorithms on a plain packed array, for the host's replay of long heap sequences:
 * the larger child is chosen by arithmetic on the comparison (no branch to mispredict on random
 * sibling orders) and an entry moves as one 8-byte copy.  Same stores, same array. */
VCU_HEAP_HD void heap_sift_up_packed(HeapEntry* h, int hole, HeapEntry v) {
    while (hole > 0) {
        const int parent = (hole - 1) >> 1;
        const HeapEntry pe = h[parent];
        if (!(pe.key < v.key)) break;
        h[hole] = pe;
        hole = parent;
    }
    h[hole] = v;
}
VCU_HEAP_HD void heap_pop_packed(HeapEntry* h, int len) {
    if (len <= 1) return;
    const int n = len - 1;
    const HeapEntry v = h[n];
    h[n] = h[0];
    int hole = 0, child = 0;
    const int lim = (n - 1) / 2;
    while (child < lim) {
        child = 2 * (child + 1);
        child -= (int)(h[child].key < h[child - 1].key);
        h[hole] = h[child];
        hole = child;
    }
    if ((n & 1) == 0 && child == (n - 2) / 2) {
        child = 2 * (child + 1);
        h[hole] = h[child - 1];
        hole = child - 1;
    }
    heap_sift_up_packed(h, hole, v);
}

/* The reference's heap sequence over a tree of regions known in stages (the control-variate waves
 * reveal which regions split, and into which children, a chunk of waves at a time): region x's
 * children are child[x] and child[x] + 1 (child[x] < 0: not known yet), key[] its error, dim[] its
 * split dimension.  run() pops the top region and pushes its two children, as
 * regions-generator-adaptive-heap.h:25-43 does, until n_splits splits are done or the top region's
 * children are not known yet; it returns that region (-1 when done) and resumes from there on the
 * next call, so replaying in stages gives the array one pass over the finished tree gives. */
struct HeapReplay {
    HeapEntry* h;        /* n_splits + 2 entries */
    size_t done = 0;     /* splits replayed */
    bool started = false;
    int run(size_t n_splits, const float* key, const int* dim, const int* child) {
        if (!started) {
            h[0] = HeapEntry{key[0], 0 | (dim[0] << 24)};
            started = true;
        }
        while (done < n_splits) {
            const int top = h[0].pay & 0xffffff;
            const int c = child[top];
            if (c < 0) return top;
            const int n = (int)done + 1;
            heap_pop_packed(h, n);
            heap_sift_up_packed(h, n - 1, HeapEntry{key[c], c | (dim[c] << 24)});
            heap_sift_up_packed(h, n, HeapEntry{key[c + 1], (c + 1) | (dim[c + 1] << 24)});
            ++done;
        }
        return -1;
    }
};

}  // namespace vcu
