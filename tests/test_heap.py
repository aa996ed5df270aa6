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
