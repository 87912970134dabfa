// ps_mma_tiles.h -- the tensor-core coupling kernels' blocks, their time steps, and the range of
// their table of B tiles, in closed form.
//
// A block of 128 pairs holds rows l1 = r0 + 2w (w = 0..3) and columns l2 = c0 + 2i (i = 0..31).
// Its skewed sweeps run nsteps(r0) time steps, in chunks of kBlk; at time step tau every pair of
// the block is at the same forward l3 and the same backward l3 (l3_at).  The B operand of a chunk
// and sweep therefore depends on the block only through the l3 of the chunk's first step, and the
// table holds one B tile per such l3 over the ranges table_geom gives.
//
// ps_mma.cu uses these definitions; tests/test_mma_tiles_host.py compiles this header with g++ and
// checks, over every block of a sweep of (lmin, lmax), that each chunk's first l3 lies in the table.
#pragma once

#include <algorithm>
#include <utility>
#include <vector>

#ifdef __CUDACC__
#define PS_MT_HD __host__ __device__
#else
#define PS_MT_HD
#endif

namespace ps_mma_tiles {

constexpr int kBlk = 32;  // time steps per chunk (one D, one fold, one pair of B tiles)

// Time steps of a block: the (2 -2 0) sweeps step one point at a time and need r0 + 68; the
// (0 0 0) sweeps step two points at a time and need floor((r0 + 1) / 2) + 34.
PS_MT_HD constexpr int nsteps(bool f00, int r0) { return f00 ? ((r0 + 1) >> 1) + 34 : r0 + 68; }

// l3 of time step tau in sweep s (0: forward, 1: backward) of the block (r0, c0).
PS_MT_HD constexpr int l3_at(bool f00, int s, int tau, int r0, int c0)
{
    return f00 ? (s ? r0 + c0 + 68 - 2 * tau : c0 - r0 - 6 + 2 * tau) : (s ? r0 + c0 + 68 - tau : c0 - r0 - 6 + tau);
}

// The table: forward tiles for first l3 = fmin .. fmin + nf - 1, then backward tiles for
// bmin .. bmin + nb - 1.  A chunk's first forward l3 is c0 - r0 - 6 plus at most r0 + 67 (the
// time steps before the block's last chunk), with r0 - 62 <= c0 <= lmax - 62: it lies in
// [-68, lmax - 1].  Its first backward l3 is r0 + c0 + 68 less the same: in [-61, 2 lmax].
struct TableGeom {
    int fmin, nf, bmin, nb;
};
PS_MT_HD constexpr TableGeom table_geom(int lmax) { return TableGeom{-72, lmax + 80, -72, 2 * lmax + 80}; }

// The blocks of one grid as (r0, c0): rows in four classes of (row parity, column parity),
// heaviest (largest r0) first.
inline void block_list(int lmin, int lmax, std::vector<std::pair<int, int>>& t)
{
    t.clear();
    for (int pr = 0; pr < 2; ++pr) {
        const int rmax = lmax - ((lmax - pr) & 1);
        for (int r0 = rmax - 6; r0 + 6 >= lmin; r0 -= 8) {
            int lo = r0;  // lowest row of the block that exists
            while (lo < lmin || lo < 0) lo += 2;
            for (int pc = 0; pc < 2; ++pc) {
                const int cmax = lmax - ((lmax - pc) & 1);
                for (int c0 = cmax - 62; c0 + 62 >= lo; c0 -= 64) t.push_back(std::make_pair(r0, c0));
            }
        }
    }
    std::stable_sort(t.begin(), t.end(), [](const std::pair<int, int>& a, const std::pair<int, int>& b) {
        return a.first > b.first;
    });
}

}  // namespace ps_mma_tiles
