"""Integrands that evaluate several points at once (pair(), multi<N>(), used by the kernels to run
independent dependency chains per lane) return exactly what operator() returns for each point.  Checked on the
host, where the same source compiles with the same explicitly rounded operations."""
import os
import subprocess
import tempfile

import numpy as np

from conftest import ROOT
from viltrum_gb300 import scenes

PROG = r'''
#include <cstdio>
#include <cstring>
#include <random>
#include <vector>
#include "vcu_integrands.h"
template <class F> int check(const F& f, int dim, int n, unsigned seed) {
    std::mt19937 rng(seed);
    std::uniform_real_distribution<float> u(-0.1f, 1.1f);
    for (int i = 0; i < n; ++i) {
        float x0[8] = {0}, x1[8] = {0}, a[3], b[3], c[3], d[3];
        for (int k = 0; k < dim; ++k) { x0[k] = u(rng); x1[k] = (i % 7 == 0) ? x0[k] : u(rng); }
        f(x0, a); f(x1, b); f.pair(x0, x1, c, d);
        if (std::memcmp(a, c, sizeof(float) * F::CH) || std::memcmp(b, d, sizeof(float) * F::CH)) {
            std::printf("mismatch at %d\n", i); return 1;
        }
    }
    return 0;
}
int main(int argc, char** argv) {
    std::vector<float> p2, p3, p5;
    FILE* fp = std::fopen(argv[1], "rb");
    int n2, n3, n5;
    if (std::fread(&n2, 4, 1, fp) != 1) return 2; p2.resize(n2); if (std::fread(p2.data(), 4, n2, fp) != (size_t)n2) return 2;
    if (std::fread(&n3, 4, 1, fp) != 1) return 2; p3.resize(n3); if (std::fread(p3.data(), 4, n3, fp) != (size_t)n3) return 2;
    if (std::fread(&n5, 4, 1, fp) != 1) return 2; p5.resize(n5); if (std::fread(p5.data(), 4, n5, fp) != (size_t)n5) return 2;
    std::fclose(fp);
    static vcu::Scene2 s2; static vcu::MovingScene3 s3; static vcu::OccludedScene5 s5;
    if (s2.build(p2.data(), n2) || s3.build(p3.data(), n3) || s5.build(p5.data(), n5)) return 3;
    int bad = check(s2, 2, 20000, 1) + check(s3, 3, 20000, 2) + check(s5, 5, 20000, 3);
    /* N-point evaluation of the scene: every point as operator() */
    std::mt19937 rng(4);
    std::uniform_real_distribution<float> u(-0.1f, 1.1f);
    for (int i = 0; i < 5000 && !bad; ++i) {
        float x[4][2], o3[3][1], o4[4][1], ref[4];
        for (int p = 0; p < 4; ++p) { x[p][0] = u(rng); x[p][1] = u(rng); s2(x[p], &ref[p]); }
        s2.multi<3>(x, o3);
        s2.multi<4>(x, o4);
        for (int p = 0; p < 4; ++p)
            if (std::memcmp(&o4[p][0], &ref[p], 4) || (p < 3 && std::memcmp(&o3[p][0], &ref[p], 4))) { bad = 1; std::printf("multi %d\n", i); }
    }
    std::printf(bad ? "bad\n" : "ok\n");
    return bad;
}
'''


def test_pair_equals_single_evaluations():
    with tempfile.TemporaryDirectory() as d:
        src, exe, prm = (os.path.join(d, n) for n in ("p.cc", "p", "params.bin"))
        open(src, "w").write(PROG)
        with open(prm, "wb") as f:
            for p in (scenes.scene2(7), scenes.moving_scene3(7), scenes.occluded_scene5(7)):
                np.array([p.size], np.int32).tofile(f)
                np.asarray(p, np.float32).tofile(f)
        subprocess.check_call(["g++", "-O2", "-std=c++17", "-ffp-contract=off", "-I", os.path.join(ROOT, "include"),
                               src, "-o", exe])
        out = subprocess.run([exe, prm], capture_output=True, text=True)
        assert out.returncode == 0 and out.stdout.strip() == "ok", out.stdout
