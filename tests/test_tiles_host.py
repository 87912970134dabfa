"""CPU checks of the chosen kernel's tiled task list (powerspectra.jl_gb300/csrc/ps_tiles.h).

The host builds the list task by task (for_each_task, used by the context
path); the allocation-free entry point fills it on the device, each row group
from its closed-form offset (group_offset over tiles_below).  A small C++
program compiled here with g++ runs both fills on the host for a sweep of
(lmin, lmax) and reports any difference; the list is also checked against a
Python statement of the tiling, and the longest list with lmax <= 4095 against
the fixed scratch of the allocation-free entry point (264192 tasks).
"""
import os
import shutil
import subprocess

import pytest

from conftest import PKG

SRC = r'''
#include <cstdio>
#include <vector>
#include "ps_tiles.h"
int main() {
    long long worst = 0, bad = 0;
    for (int lmax = 0; lmax <= 4095; lmax += (lmax < 300 ? 1 : 97)) {
        for (int lmin = 0; lmin <= lmax; lmin += (lmax - lmin < 70 ? 1 : 61)) {
            std::vector<long long> a, b;
            ps_tiles::for_each_task(lmin, lmax, [&](int l1, int l2) { a.push_back(((long long)l1 << 32) ^ (unsigned)l2); });
            const ps_tiles::Geometry G = ps_tiles::geometry(lmin, lmax);
            const long long n = ps_tiles::task_count(lmin, lmax);
            b.assign((size_t)n, -7);
            for (int g = G.glo; g < 8 * G.nb; ++g) {   /* the device fill, one row group at a time */
                long long t = ps_tiles::group_offset(G, g);
                for (int c = g / 8; c < G.nb; ++c)
                    for (int q = 0; q < 4; ++q, ++t) {
                        const int l1 = G.o + 4 * g + q;
                        if (t < 0 || t >= n) { ++bad; continue; }
                        b[(size_t)t] = ((long long)(l1 >= lmin ? l1 : -1) << 32) ^ (unsigned)(G.o + 32 * c);
                    }
            }
            if ((long long)a.size() != n || a != b) { ++bad; std::printf("MISMATCH %d %d\n", lmin, lmax); }
            if (n > worst) worst = n;
        }
    }
    std::printf("%lld %lld %lld\n", bad, worst, ps_tiles::task_count(0, 4095));
    return 0;
}
'''


@pytest.fixture(scope="module")
def sweep(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("tiles")
    src, exe = os.path.join(d, "t.cpp"), os.path.join(d, "t")
    open(src, "w").write(SRC)
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(PKG, "csrc"), src, "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True).stdout.split()
    return [int(x) for x in out[-3:]], out


def test_device_fill_matches_host_list(sweep):
    (bad, _, _), out = sweep
    assert bad == 0, out[:20]


def test_longest_list_fits_the_fixed_scratch(sweep):
    (_, worst, full), _ = sweep
    assert full == 264192
    assert worst <= full


def _python_tiles(lmin, lmax):
    n = lmax - lmin + 1
    nb = (n + 31) // 32
    o = lmax + 1 - 32 * nb
    out = []
    for g in range(8 * nb - 1, (lmin - o) // 4 - 1, -1):
        for b in range(g // 8, nb):
            for q in range(4):
                l1 = o + 4 * g + q
                out.append((l1 if l1 >= lmin else -1, o + 32 * b))
    return out


@pytest.mark.parametrize("lmin,lmax", [(0, 0), (0, 31), (3, 40), (0, 767), (17, 300), (2, 1000)])
def test_tiles_cover_every_pair_once(lmin, lmax):
    """Every (l1 <= l2) pair of the grid lies in exactly one task's 32 columns."""
    seen = {}
    for (l1, l2_0) in _python_tiles(lmin, lmax):
        if l1 < 0:
            continue
        for l2 in range(l2_0, l2_0 + 32):
            if l1 <= l2 <= lmax:
                seen[l1, l2] = seen.get((l1, l2), 0) + 1
    want = {(a, b) for a in range(lmin, lmax + 1) for b in range(a, lmax + 1)}
    assert set(seen) == want and set(seen.values()) == {1}
