"""The culled evaluation of the scene (multi_cull: only the terms that can be non-zero in a box)
returns exactly what operator() returns at every point of the box -- checked on the host, where the
same source compiles with the same explicitly rounded operations: boxes from 1/2048 of the square
(finer than the benchmark's bins) to the whole square, at the origin and far from it, points drawn inside, on the edges and at the
corners, and the node coordinates a nested rule places there."""
import os
import subprocess

import numpy as np

from conftest import ROOT
from viltrum_gb300 import scenes

PROG = r'''
#include <cstdio>
#include <cstdlib>
#include <cstring>
#include <random>
#include <vector>
#include "vcu_integrands.h"
int main(int argc, char** argv) {
    std::vector<float> p;
    FILE* fp = std::fopen(argv[1], "rb");
    int n;
    if (std::fread(&n, 4, 1, fp) != 1) return 2;
    p.resize(n);
    if (std::fread(p.data(), 4, n, fp) != (size_t)n) return 2;
    std::fclose(fp);
    const float off = (float)std::atof(argv[2]);
    static vcu::Scene2 s;
    if (s.build(p.data(), n)) return 3;
    std::mt19937 rng(5);
    std::uniform_real_distribution<float> u01(0.0f, 1.0f);
    long kept = 0, terms = 0, checked = 0;
    const float widths[] = {1.0f / 2048, 1.0f / 512, 1.0f / 64, 1.0f / 8, 1.0f};
    for (float w : widths) {
        for (int b = 0; b < 2000; ++b) {
            float lo[2], hi[2];
            for (int k = 0; k < 2; ++k) {
                const int cells = (int)(1.0f / w);
                const int pos = (int)(u01(rng) * cells) % (cells > 0 ? cells : 1);
                lo[k] = vcu::vadd(off, vcu::vmul((float)pos, w));
                hi[k] = vcu::vadd(off, vcu::vmul((float)(pos + 1), w));
            }
            const auto c = s.cull(lo, hi);
            kept += __builtin_popcountll(c.g) + __builtin_popcount(c.d);
            terms += s.ng + s.nd;
            for (int q = 0; q < 24; ++q) {
                float x[4][2];
                for (int t = 0; t < 4; ++t)
                    for (int k = 0; k < 2; ++k) {
                        const int mode = (q + t + k) % 6;
                        /* inside, edges, corners, Boole's node positions */
                        const float v = mode == 0 ? lo[k] : mode == 1 ? hi[k]
                                      : mode == 2 ? vcu::vadd(lo[k], vcu::vmul(0.25f, vcu::vsub(hi[k], lo[k])))
                                      : mode == 3 ? vcu::vadd(lo[k], vcu::vmul(0.75f, vcu::vsub(hi[k], lo[k])))
                                      : vcu::vadd(lo[k], vcu::vmul(u01(rng), vcu::vsub(hi[k], lo[k])));
                        x[t][k] = v;
                    }
                float o[4][1];
                s.multi_cull<4>(c, x, o);
                for (int t = 0; t < 4; ++t) {
                    float r[1];
                    s(x[t], r);
                    ++checked;
                    if (std::memcmp(r, o[t], 4)) {
                        std::printf("mismatch w=%g box [%a,%a]x[%a,%a] at (%a,%a): %a vs %a\n", w, lo[0], hi[0],
                                    lo[1], hi[1], x[t][0], x[t][1], r[0], o[t][0]);
                        return 1;
                    }
                }
            }
        }
    }
    std::printf("%ld %ld %ld\n", checked, kept, terms);
    return 0;
}
'''


def test_culled_scene_equals_full_evaluation(tmp_path):
    src = tmp_path / "cull.cc"
    src.write_text(PROG)
    exe = tmp_path / "cull"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True)
    # the scene over [0,1]^2, and moved to [100,101]^2 where a coordinate's ulp is 8e-6
    for seed, off in ((7, 0.0), (3, 0.0), (7, 100.0)):
        p = np.asarray(scenes.scene2(seed), np.float32)
        ng, nd = int(p[0]), int(p[1])
        for base in [2 + 4 * i for i in range(ng + nd)]:
            p[base:base + 2] += np.float32(off)
        f = tmp_path / f"p{seed}_{int(off)}.bin"
        with open(f, "wb") as fh:
            fh.write(np.int32(p.size).tobytes())
            fh.write(p.tobytes())
        r = subprocess.run([str(exe), str(f), str(off)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        checked, kept, terms = (int(x) for x in r.stdout.split())
        assert checked == 5 * 2000 * 24 * 4 and kept < terms  # something is culled


COUNT = r'''
#include <cstdio>
#include <vector>
#include "vcu_integrands.h"
int main(int argc, char** argv) {
    std::vector<float> p;
    FILE* fp = std::fopen(argv[1], "rb");
    int n;
    if (std::fread(&n, 4, 1, fp) != 1) return 2;
    p.resize(n);
    if (std::fread(p.data(), 4, n, fp) != (size_t)n) return 2;
    std::fclose(fp);
    static vcu::Scene2 s;
    if (s.build(p.data(), n)) return 3;
    const int res = 128;
    double flops = 0.0;
    for (int j = 0; j < res; ++j)
        for (int i = 0; i < res; ++i) {
            const float lo[2] = {vcu::vmul((float)i, 1.0f / res), vcu::vmul((float)j, 1.0f / res)};
            const float hi[2] = {vcu::vmul((float)(i + 1), 1.0f / res), vcu::vmul((float)(j + 1), 1.0f / res)};
            const auto c = s.cull(lo, hi);
            flops += 31.0 * __builtin_popcountll(c.g) + 6.0 * __builtin_popcount(c.d);
        }
    std::printf("%.6f\n", flops / (res * res));
    return 0;
}
'''


def test_benchmark_flop_count_matches_the_cull(tmp_path):
    """The benchmark's roofline counts the flops of the terms a bin keeps (bench.culled_flops_per_eval,
    exact geometry); the device's conservative cull keeps at least those and only slightly more."""
    import bench

    src = tmp_path / "count.cc"
    src.write_text(COUNT)
    exe = tmp_path / "count"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True)
    p = np.asarray(scenes.scene2(7), np.float32)
    f = tmp_path / "p.bin"
    with open(f, "wb") as fh:
        fh.write(np.int32(p.size).tobytes())
        fh.write(p.tobytes())
    r = subprocess.run([str(exe), str(f)], capture_output=True, text=True, check=True)
    device = float(r.stdout)
    model = bench.culled_flops_per_eval(p, [0, 0], [1, 1], [128, 128])
    assert model <= device <= model * 1.01, (model, device)


OCCLUDED = r'''
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>
#include "vcu_integrands.h"
int main(int argc, char** argv) {
    std::vector<float> p;
    FILE* fp = std::fopen(argv[1], "rb");
    int n;
    if (std::fread(&n, 4, 1, fp) != 1) return 2;
    p.resize(n);
    if (std::fread(p.data(), 4, n, fp) != (size_t)n) return 2;
    std::fclose(fp);
    static vcu::OccludedScene5 s;
    if (s.build(p.data(), n)) return 3;
    std::mt19937 rng(9);
    std::uniform_real_distribution<float> u01(0.0f, 1.0f);
    long checked = 0, zero = 0;
    for (int res : {1024, 64, 8}) {
        const float w = 1.0f / (float)res;
        for (int b = 0; b < 1500; ++b) {
            const int ix = (int)(u01(rng) * res) % res, iy = (int)(u01(rng) * res) % res;
            const float lo[2] = {vcu::vmul((float)ix, w), vcu::vmul((float)iy, w)};
            const float wx = vcu::vsub(vcu::vmul((float)(ix + 1), w), lo[0]);
            const float wy = vcu::vsub(vcu::vmul((float)(iy + 1), w), lo[1]);
            const float hi[2] = {vcu::vadd(lo[0], wx), vcu::vadd(lo[1], wy)};
            const auto c = s.cull_box(lo, hi);
            for (int q = 0; q < 16; ++q) {
                float x0[5], x1[5];
                /* as the per-bin Monte Carlo kernel draws them: u * width + lo */
                x0[0] = vcu::vadd(vcu::vmul(u01(rng), wx), lo[0]);
                x0[1] = vcu::vadd(vcu::vmul(u01(rng), wy), lo[1]);
                x1[0] = q & 1 ? lo[0] : hi[0];
                x1[1] = q & 2 ? lo[1] : hi[1];
                for (int k = 2; k < 5; ++k) {
                    x0[k] = u01(rng);
                    x1[k] = u01(rng);
                }
                float a0[1], a1[1], b0[1], b1[1], r0[1], r1[1];
                s.pair_culled(c, x0, x1, a0, a1);
                s.pair(x0, x1, b0, b1);
                s(x0, r0);
                s(x1, r1);
                checked += 2;
                zero += (r0[0] == 0.0f) + (r1[0] == 0.0f);
                if (std::memcmp(a0, r0, 4) || std::memcmp(a1, r1, 4) || std::memcmp(b0, r0, 4) || std::memcmp(b1, r1, 4)) {
                    std::printf("mismatch res=%d bin (%d,%d): %a %a %a | %a %a %a\n", res, ix, iy, r0[0], a0[0], b0[0],
                                r1[0], a1[0], b1[0]);
                    return 1;
                }
            }
        }
    }
    std::printf("%ld %ld\n", checked, zero);
    return 0;
}
'''


def test_occluded_scene_culled_pair_equals_full_evaluation(tmp_path):
    """The occluded 5-D scene's pair_culled (only the scene terms that can be non-zero over a bin's box
    of the first two coordinates) and its pair (which skips the visibility of a point whose scene
    value is 0) return what operator() returns, bit for bit, at points drawn inside the bins and at
    their corners."""
    src = tmp_path / "occ.cc"
    src.write_text(OCCLUDED)
    exe = tmp_path / "occ"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True)
    p = np.asarray(scenes.occluded_scene5(7), np.float32)
    f = tmp_path / "occ.bin"
    with open(f, "wb") as fh:
        fh.write(np.int32(p.size).tobytes())
        fh.write(p.tobytes())
    r = subprocess.run([str(exe), str(f)], capture_output=True, text=True)
    assert r.returncode == 0, r.stdout + r.stderr
    checked, zero = (int(x) for x in r.stdout.split())
    assert checked == 3 * 1500 * 16 * 2 and 0 < zero < checked


MOVING = r'''
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>
#include "vcu_integrands.h"
int main(int argc, char** argv) {
    std::vector<float> p;
    FILE* fp = std::fopen(argv[1], "rb");
    int n;
    if (std::fread(&n, 4, 1, fp) != 1) return 2;
    p.resize(n);
    if (std::fread(p.data(), 4, n, fp) != (size_t)n) return 2;
    std::fclose(fp);
    static vcu::MovingScene3 s;
    if (s.build(p.data(), n)) return 3;
    std::mt19937 rng(11);
    std::uniform_real_distribution<float> u01(0.0f, 1.0f);
    long checked = 0, kept = 0, terms = 0;
    for (int res : {512, 64, 8}) {
        for (int tcut : {1, 4}) { /* the whole of t, or a quarter of it */
            const float w = 1.0f / (float)res;
            for (int b = 0; b < 1500; ++b) {
                const int ix = (int)(u01(rng) * res) % res, iy = (int)(u01(rng) * res) % res;
                const int it = (int)(u01(rng) * tcut) % tcut;
                const float lo[3] = {vcu::vmul((float)ix, w), vcu::vmul((float)iy, w), vcu::vmul((float)it, 1.0f / tcut)};
                const float hi[3] = {vcu::vmul((float)(ix + 1), w), vcu::vmul((float)(iy + 1), w),
                                     vcu::vmul((float)(it + 1), 1.0f / tcut)};
                const auto c = s.cull_box(lo, hi);
                kept += __builtin_popcountll(c.g) + __builtin_popcount(c.d);
                terms += s.ng + s.nd;
                for (int q = 0; q < 16; ++q) {
                    float x[3];
                    for (int k = 0; k < 3; ++k) {
                        const int mode = (q + k) % 4; /* inside, or on either face */
                        x[k] = mode == 0 ? lo[k] : mode == 1 ? hi[k]
                             : vcu::vadd(lo[k], vcu::vmul(u01(rng), vcu::vsub(hi[k], lo[k])));
                    }
                    float a[3], r[3], y[3], pa[3], pb[3], ry[3];
                    s.eval_culled(c, x, a);
                    s(x, r);
                    /* a second point of the box with the first, through pair_culled */
                    for (int k = 0; k < 3; ++k) y[k] = vcu::vadd(lo[k], vcu::vmul(u01(rng), vcu::vsub(hi[k], lo[k])));
                    s.pair_culled(c, x, y, pa, pb);
                    s(y, ry);
                    ++checked;
                    if (std::memcmp(a, r, sizeof(a)) || std::memcmp(pa, r, sizeof(pa)) || std::memcmp(pb, ry, sizeof(pb))) {
                        std::printf("mismatch res=%d at (%a,%a,%a)\n", res, x[0], x[1], x[2]);
                        return 1;
                    }
                }
            }
        }
    }
    std::printf("%ld %ld %ld\n", checked, kept, terms);
    return 0;
}
'''


def test_moving_scene_culled_evaluation_equals_full_evaluation(tmp_path):
    """The moving-disk scene's eval_culled and pair_culled (bumps culled as in the 2-D scene, disks by
    their centre's path over the box's time interval) return operator()'s three channels bit for bit
    at points of the box, for bins of 1/512 to 1/8 and the whole or a quarter of the time range."""
    src = tmp_path / "mov.cc"
    src.write_text(MOVING)
    exe = tmp_path / "mov"
    subprocess.run(["g++", "-std=c++17", "-O2", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"), str(src),
                    "-o", str(exe)], check=True)
    for seed in (7, 3):
        p = np.asarray(scenes.moving_scene3(seed), np.float32)
        f = tmp_path / f"mov{seed}.bin"
        with open(f, "wb") as fh:
            fh.write(np.int32(p.size).tobytes())
            fh.write(p.tobytes())
        r = subprocess.run([str(exe), str(f)], capture_output=True, text=True)
        assert r.returncode == 0, r.stdout + r.stderr
        checked, kept, terms = (int(x) for x in r.stdout.split())
        assert checked == 3 * 2 * 1500 * 16 and kept < terms
