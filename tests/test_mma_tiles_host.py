"""CPU checks of the tensor-core kernels' blocks and their table of B tiles
(powerspectra.jl_gb300/csrc/ps_mma_tiles.h).

Each 32-step chunk of a block copies two tiles from the table: the forward one of the chunk's
first forward l3 and the backward one of its first backward l3.  A small C++ program compiled
here with g++ walks every chunk of every block for a sweep of (lmin, lmax) and both families, and
reports any first l3 outside the table's ranges, along with the extremes it saw, which must lie
in the ranges the header derives: forward [-68, lmax - 1], backward [-61, 2 lmax].  The blocks
are also checked to cover every pair (l1 <= l2) of the grid exactly once.
"""
import os
import shutil
import subprocess

import pytest

from conftest import PKG

SRC = r'''
#include <cstdio>
#include <vector>
#include "ps_mma_tiles.h"
using namespace ps_mma_tiles;
int main() {
    long long bad = 0, chunks = 0, outside = 0;
    std::vector<std::pair<int, int>> t;
    std::vector<int> lmaxes;
    for (int l = 0; l <= 300; ++l) lmaxes.push_back(l);
    for (int l = 301; l <= 4200; l += 37) lmaxes.push_back(l);
    for (int l : {6143, 8191, 12288, 16383}) lmaxes.push_back(l);
    for (int lmax : lmaxes) {
        const TableGeom G = table_geom(lmax);
        for (int lmin = 0; lmin <= lmax; lmin += (lmax - lmin < 40 ? 1 : (lmax > 4200 ? lmax / 3 : 53))) {
            block_list(lmin, lmax, t);
            // every pair of the grid in exactly one block (small grids)
            if (lmax <= 160) {
                std::vector<int> seen((size_t)(lmax + 1) * (lmax + 1), 0);
                for (auto& b : t)
                    for (int w = 0; w < 4; ++w)
                        for (int i = 0; i < 32; ++i) {
                            const int l1 = b.first + 2 * w, l2 = b.second + 2 * i;
                            if (l1 >= lmin && l1 <= lmax && l2 >= l1 && l2 <= lmax) ++seen[(size_t)l1 * (lmax + 1) + l2];
                        }
                for (int l1 = lmin; l1 <= lmax; ++l1)
                    for (int l2 = l1; l2 <= lmax; ++l2)
                        if (seen[(size_t)l1 * (lmax + 1) + l2] != 1) { ++bad; std::printf("COVER %d %d %d %d\n", lmin, lmax, l1, l2); }
            }
            for (int f00 = 0; f00 < 2; ++f00)
                for (auto& b : t) {
                    const int nk = (nsteps(f00, b.first) + kBlk - 1) / kBlk;
                    for (int q = 0; q < nk; ++q) {
                        if (lmax > 4200 && q > 0 && q < nk - 1) continue;  // the first l3 is monotone in q
                        ++chunks;
                        const int of = l3_at(f00, 0, q * kBlk, b.first, b.second);
                        const int ob = l3_at(f00, 1, q * kBlk, b.first, b.second);
                        if (of < G.fmin || of >= G.fmin + G.nf || ob < G.bmin || ob >= G.bmin + G.nb) {
                            ++bad;
                            std::printf("TABLE %d %d %d %d %d %d %d\n", f00, lmin, lmax, b.first, b.second, of, ob);
                        }
                        if (of < -68 || of > lmax - 1 || ob < -61 || ob > 2 * lmax) ++outside;
                    }
                }
        }
    }
    std::printf("%lld %lld %lld\n", bad, outside, chunks);
    return 0;
}
'''


@pytest.fixture(scope="module")
def walk(tmp_path_factory):
    gxx = shutil.which("g++")
    if not gxx:
        pytest.skip("g++ not available")
    d = tmp_path_factory.mktemp("mma_tiles")
    src, exe = os.path.join(d, "t.cpp"), os.path.join(d, "t")
    open(src, "w").write(SRC)
    subprocess.run([gxx, "-std=c++17", "-O2", "-I", os.path.join(PKG, "csrc"), src, "-o", exe], check=True)
    out = subprocess.run([exe], check=True, capture_output=True, text=True, timeout=600).stdout.split()
    return [int(x) for x in out[-3:]], out


def test_every_chunk_reads_inside_the_table(walk):
    (bad, _, chunks), out = walk
    assert chunks > 10**6
    assert bad == 0, out[:40]


def test_first_l3_within_the_derived_ranges(walk):
    (_, outside, _), _ = walk
    assert outside == 0
