"""The device heap (viltrum_gb300/csrc/vcu_heap.h) makes libstdc++'s choices: the two-array form,
the packed-entry form over one array and split between two (as the batched kernel keeps its top
levels in shared memory), and the branch-free packed form the host replays long sequences with.

A small host program drives vcu::heap_push / heap_pop and std::push_heap / std::pop_heap with
the same random sequences (with many equal keys, which is where the two could disagree) and
compares the full arrays after every operation."""
import os
import subprocess
import tempfile

from conftest import ROOT

PROG = r'''
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>
#include "vcu_heap.h"
struct E { float k; int p; };
int main() {
    std::mt19937 rng(1);
    for (int trial = 0; trial < 400; ++trial) {
        std::vector<E> ref;
        float key[128]; int pay[128]; int n = 0; int next = 0;
        vcu::HeapEntry one[130], top[16], rest[130], flat[130];
        const vcu::HeapArray ha{one};
        const vcu::HeapSplit hs{top, rest, 7};
        const int levels = 1 + trial % 7;
        for (int op = 0; op < 300; ++op) {
            const bool push = n == 0 || (n < 120 && (rng() % 3) != 0);
            if (push) {
                const float k = float(rng() % levels);
                ref.push_back({k, next});
                std::push_heap(ref.begin(), ref.end(), [](const E& a, const E& b) { return a.k < b.k; });
                key[n] = k; pay[n] = next; ++n; ++next;
                vcu::heap_push(key, pay, n);
                ha.set(n - 1, vcu::HeapEntry{k, next - 1});
                vcu::heap_push_entries(ha, n);
                hs.set(n - 1, vcu::HeapEntry{k, next - 1});
                vcu::heap_push_entries(hs, n);
                vcu::heap_sift_up_packed(flat, n - 1, vcu::HeapEntry{k, next - 1});
            } else {
                std::pop_heap(ref.begin(), ref.end(), [](const E& a, const E& b) { return a.k < b.k; });
                ref.pop_back();
                vcu::heap_pop(key, pay, n);
                vcu::heap_pop_entries(ha, n);
                vcu::heap_pop_entries(hs, n);
                vcu::heap_pop_packed(flat, n); --n;
            }
            for (int i = 0; i < n; ++i)
                if (ref[i].k != key[i] || ref[i].p != pay[i] || ref[i].k != ha.get(i).key || ref[i].p != ha.get(i).pay ||
                    ref[i].k != hs.get(i).key || ref[i].p != hs.get(i).pay || ref[i].k != flat[i].key ||
                    ref[i].p != flat[i].pay) {
                    std::printf("mismatch trial %d op %d\n", trial, op); return 1; }
        }
    }
    std::printf("ok\n");
    return 0;
}
'''


def test_heap_matches_libstdcxx():
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "h.cc")
        exe = os.path.join(d, "h")
        open(src, "w").write(PROG)
        subprocess.check_call(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "viltrum_gb300", "csrc"), src,
                               "-o", exe])
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout
        assert out.stdout.strip() == "ok"


PROG_STAGED = r"""
#include <algorithm>
#include <cstdio>
#include <random>
#include <vector>
#include "vcu_heap.h"
/* A tree of regions grown as the sequence needs it (errors decaying with depth, many equal), plus
 * splits the sequence never uses (the waves' overshoot); its children then revealed in random
 * batches.  HeapReplay, run batch by batch, against std::pop_heap / std::push_heap in one pass. */
int main() {
    std::mt19937 rng(3);
    int compared = 0;
    for (int trial = 0; trial < 200; ++trial) {
        const int N = 50 + (int)(rng() % 3000); /* splits */
        const int extra = (int)(rng() % 400);   /* splits no pop reaches */
        const int pool = 2 * (N + extra) + 1;
        const int levels = 1 + trial % 5;
        std::vector<float> key(pool);
        std::vector<int> dim(pool), child(pool, -1);
        key[0] = 1.0f;
        int next = 1;
        auto split = [&](int x) {
            child[x] = next;
            for (int c = 0; c < 2; ++c) {
                key[next + c] = key[x] * (float)(1 + rng() % levels) / (float)(levels + 1);
                dim[next + c] = (int)(rng() % 5);
            }
            next += 2;
        };
        /* the one-pass sequence with libstdc++, splitting each region when it is popped */
        struct E { float k; int p; };
        auto less = [](const E& a, const E& b) { return a.k < b.k; };
        std::vector<E> ref{{key[0], 0 | (dim[0] << 24)}};
        for (int it = 0; it < N; ++it) {
            const int top = ref[0].p & 0xffffff;
            if (child[top] < 0) split(top);
            const int c = child[top];
            std::pop_heap(ref.begin(), ref.end(), less);
            ref.back() = {key[c], c | (dim[c] << 24)};
            std::push_heap(ref.begin(), ref.end(), less);
            ref.push_back({key[c + 1], (c + 1) | (dim[c + 1] << 24)});
            std::push_heap(ref.begin(), ref.end(), less);
        }
        /* overshoot: split some regions still in the heap */
        for (int q = 0; q < extra; ++q) {
            const int x = ref[rng() % ref.size()].p & 0xffffff;
            if (child[x] < 0 && next + 2 <= pool) split(x);
        }
        /* staged: children hidden, revealed in random batches */
        std::vector<int> shown(pool, -1), order;
        for (int x = 0; x < next; ++x)
            if (child[x] >= 0) order.push_back(x);
        std::shuffle(order.begin(), order.end(), rng);
        std::vector<vcu::HeapEntry> h(N + 2);
        vcu::HeapReplay rp{h.data()};
        size_t at = 0;
        int stages = 0;
        int missing = rp.run(N, key.data(), dim.data(), shown.data());
        while (missing >= 0) {
            if (at == order.size()) { std::printf("stuck trial %d\n", trial); return 1; }
            const size_t batch = 1 + rng() % 64;
            for (size_t q = 0; q < batch && at < order.size(); ++q, ++at) shown[order[at]] = child[order[at]];
            missing = rp.run(N, key.data(), dim.data(), shown.data());
            ++stages;
        }
        for (int i = 0; i <= N; ++i)
            if (h[i].key != ref[i].k || h[i].pay != ref[i].p) { std::printf("mismatch trial %d at %d\n", trial, i); return 1; }
        compared += stages > 1;
    }
    std::printf("ok %d\n", compared);
    return 0;
}
"""


def test_staged_replay_matches_one_pass():
    """The control-variate generator replays the heap sequence while later waves are still running:
    HeapReplay pauses at a region whose children are not known yet and resumes when they are.  Over
    random trees (decaying errors with many ties) whose splits are revealed in random batches, the
    final array equals libstdc++'s one-pass push_heap / pop_heap sequence."""
    with tempfile.TemporaryDirectory() as d:
        src = os.path.join(d, "s.cc")
        exe = os.path.join(d, "s")
        open(src, "w").write(PROG_STAGED)
        subprocess.check_call(["g++", "-O1", "-std=c++17", "-I", os.path.join(ROOT, "viltrum_gb300", "csrc"), src,
                               "-o", exe])
        out = subprocess.run([exe], capture_output=True, text=True)
        assert out.returncode == 0, out.stdout
        word, staged = out.stdout.split()
        assert word == "ok" and int(staged) >= 150, out.stdout  # trials that paused and resumed
