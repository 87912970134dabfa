// ps_tiles.h -- the chosen coupling kernel's tiled task list, in closed form.
//
// A task is (l1, l2_0): one warp's 32 consecutive l2 of row l1.  The list is
// tiled for blocks of four warps: with n = lmax - lmin + 1, nb = ceil(n / 32)
// and o = lmax + 1 - 32 nb (so that the last 32-column block ends at lmax),
// tile (g, b) holds rows o + 4g .. o + 4g + 3 (l1 = -1 for rows below lmin)
// over the 32 columns from o + 32 b, for b = g / 8 .. nb - 1.  Row groups run
// from the top (g = 8 nb - 1, the longest families) down to glo = (lmin - o) / 4.
// Every row then has the warp tasks that 32-column steps from l1 would give,
// and the only idle lanes are those left of the diagonal.
//
// The host builds the list with for_each_task (ps_api.cu); the
// allocation-free entry point fills it on the device from group_offset
// (ps_noalloc.cu); tests/test_tiles_host.py checks that both give the same
// tasks in the same order.  Plain C++17, so the CPU test compiles it with g++.
#pragma once

#ifdef __CUDACC__
#define PS_TILES_HD __host__ __device__
#else
#define PS_TILES_HD
#endif

namespace ps_tiles {

struct Geometry {
    int n, nb, o, glo;  // rows, 32-column blocks, first row / column of the tiling, lowest row group
};

PS_TILES_HD constexpr Geometry geometry(int lmin, int lmax)
{
    const int n = lmax - lmin + 1, nb = (n + 31) / 32, o = lmax + 1 - 32 * nb;
    return Geometry{n, nb, o, (lmin - o) / 4};
}

// Tiles of row groups 0 .. m - 1: the sum of nb - g / 8 over g < m.
PS_TILES_HD constexpr long long tiles_below(long long m, long long nb)
{
    const long long q = m / 8, r = m % 8;
    return m * nb - (4 * q * (q - 1) + r * q);
}

// Number of tasks (four per tile) of the list for (lmin, lmax).
PS_TILES_HD constexpr long long task_count(int lmin, int lmax)
{
    const Geometry G = geometry(lmin, lmax);
    return 4 * (tiles_below(8LL * G.nb, G.nb) - tiles_below(G.glo, G.nb));
}

// Index of the first task of row group g (groups above g come first).
PS_TILES_HD constexpr long long group_offset(const Geometry& G, int g)
{
    return 4 * (tiles_below(8LL * G.nb, G.nb) - tiles_below(g + 1, G.nb));
}

// The tasks in list order: emit(l1, l2_0) with l1 = -1 for rows below lmin.
template <typename Emit>
inline void for_each_task(int lmin, int lmax, Emit emit)
{
    const Geometry G = geometry(lmin, lmax);
    for (int g = 8 * G.nb - 1; g >= G.glo; --g)
        for (int b = g / 8; b < G.nb; ++b)
            for (int q = 0; q < 4; ++q) {
                const int l1 = G.o + 4 * g + q;
                emit(l1 >= lmin ? l1 : -1, G.o + 32 * b);
            }
}

}  // namespace ps_tiles
