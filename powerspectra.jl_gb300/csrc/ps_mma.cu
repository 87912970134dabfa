// ps_mma.cu -- coupling kernels for sets of windows with the window
// contraction on the tensor cores (tcgen05, BF16 in, FP32 out).
//
// One launch computes up to 15 windows of one family product with ONE
// generation of the family per pair, where the chosen kernel contracts at most
// 8 windows per generation on the CUDA cores:
//   * the (2 -2 0) family squared, with each window's parity of l1 + l2 + l3:
//     M++ (EE/BB diagonal blocks, even), M-- (off-diagonal, odd) and the
//     all-parity Xi (src/modecoupling.jl:123-159 per window);
//   * the (0 0 0) family squared: M00, TT (src/modecoupling.jl:78-95).
// (src/covariance.jl:92-183 contracts 8 windows against one family.)
//
// Mapping.  A block holds 4 rows l1 = r0 + 2w (one per warp) and 32 columns
// l2 = c0 + 2i (one per lane): 128 pairs, the M = 128 rows of the MMA.  The
// sweeps run in registers in float-float arithmetic as in the chosen kernel,
// but time-skewed: at time step tau, lane (w, i) takes forward step
// tF = tau - 6 - 2i + 2w (point l3 = l2 - l1 + tF) and backward step
// tB = tau + 2w + 2i - 68 (point l3 = l1 + l2 - tB).  Then every pair of the
// block is at the same forward l3 = c0 - r0 - 6 + tau and the same backward
// l3 = r0 + c0 + 68 - tau, and every step has the parity of tau, so the
// contraction over one block of 16 time steps is a dense product
//     D[pair, slot] = sum_tau x[pair, tau] B[tau, slot],
// x = f^2 (the family value squared) and B = the windows at that tau, with the
// parity of each slot applied to B's rows.  A 16th column of B holds 2 l3 + 1
// and gives the normalisation sum.  Each lane runs at most 68 idle steps at
// the ramps (lanes start and finish at different tau).
//
// The (0 0 0) family vanishes where l1 + l2 + l3 is odd, so its sweeps step two
// points per time step: lane (w, i) takes forward step nF = tau - i + w - 3
// (l3 = l2 - l1 + 2 nF) and backward step nB = tau + w + i - 34
// (l3 = l1 + l2 - 2 nB); every pair is at forward l3 = c0 - r0 - 6 + 2 tau and
// backward l3 = r0 + c0 + 68 - 2 tau: half the time steps of the one-point
// skew.
//
// Precision.  x and B are split into three BF16 parts (hi + mid + lo carries
// 24 bits) and D is formed from six products (all but the three smallest),
// ordered so that the hi x hi products are added last: the tensor core rounds
// its FP32 accumulation toward zero, so each block's D starts from zero and
// takes such a rounding at full scale only for the hi x hi of each of its two
// MMA halves: the second onto the first (at twice the scale) or, with at most
// 8 columns, in D's spare columns on its own.  Each D is added to float-float
// totals on the CUDA cores (into the low word; renormalised every fourth
// block).  B holds each column scaled by the largest power of two of its values
// in the block (block floating point; windows span 1e-45), the same role the
// slice exponents play in the chosen kernel; the fold brings D to the totals'
// running exponent.  The last forward point, the match of the two sweeps, the
// normalisation and the outputs are FP64.
//
// B tiles.  B of one block and sweep depends on the block's position only
// through o, the l3 of its first time step: its step k holds the windows at
// l3 = o + k (forward) or o - k (backward), o + 2k and o - 2k for the (0 0 0)
// sweeps, with the slots' parities by the parity of k.  So a table kernel
// builds, before the coupling kernel, one B tile per o that the launch's blocks
// use, and a block takes its two tiles with two bulk copies.
//
// Pipeline per block q of 32 time steps: at its start the lanes build the
// block's new ring values, wait (bounded) for the MMAs of block q - 1 and add
// its D into the totals; one thread starts the copies of block q + 1's tiles
// into the buffer that those MMAs have released, and the last warp takes block
// q's column scales from its tiles (copied a block ahead).  Then the lanes
// write x (three planes, two steps per 32-bit column, two MMA halves) into
// tensor memory, and at the block end two threads (one per sweep, in
// different warps) issue the 24 MMAs of q, 12 each, and commit them to one
// mbarrier.  A and D are single-buffered (128 tensor memory columns per
// block), B double-buffered in shared memory.  A wait that gives up sets
// *p.status.
#include "ps_internal.cuh"
#include "ps_epilogue.cuh"
#include "ps_ff.cuh"
#include "ps_umma.cuh"
#include "ps_mma_tiles.h"

#include <cuda_bf16.h>
#include <algorithm>
#include <type_traits>
#include <vector>

namespace ps {
namespace {

constexpr int kK = 16;            // time steps per MMA (BF16 K)
constexpr int kBlk = ps_mma_tiles::kBlk;  // time steps per block: two MMA halves, one D, one barrier
static_assert(kBlk == 2 * kK, "a block is two MMA halves");
constexpr int kPlanes = 3;        // hi, mid, lo BF16 parts
constexpr int kLead = 6;          // forward skew offset: tF = tau - kLead - 2i + 2w
constexpr int kRamp = 68;         // extra time steps of a block beyond r0 (both sweeps)
// From tau = kSteady to tau = r0 + kLead - 1 every lane of the block that runs is inside both of
// its sweeps: the forward sweep of lane (w, i) spans tau = 6 + 2i - 2w .. r0 + 5 + 2i and the
// backward one tau = 68 - 2w - 2i .. r0 + 67 - 2i.
constexpr int kSteady = 68;
constexpr uint32_t kTmemCols = 128;
constexpr int kBPlane = kMmaCols * kK * 2;  // bytes of one BF16 B plane: 16 columns x 16 steps
constexpr int kWaitLimit = 1 << 22;
constexpr uint32_t kIdesc = umma::idesc_bf16(128, kMmaCols);
// six of the nine products of the three-part split, small first, hi x hi last:
// (A part, B part)
__device__ constexpr int kPass[6][2] = {{2, 0}, {1, 1}, {0, 2}, {1, 0}, {0, 1}, {0, 0}};

// tensor memory columns: D forward [0, 16), D backward [16, 32), then A[sweep][plane][half], 8
// columns per half: a block's 32 steps of one sweep and plane in 16 consecutive columns, two
// steps per column (step pair k of the block in column a_col(s, p) + k)
__device__ __forceinline__ uint32_t a_col(int sweep, int plane, int half = 0)
{
    return 2u * kMmaCols + (uint32_t)(((sweep * kPlanes + plane) * 2 + half) * (kK / 2));
}

// B of one block and sweep, as the table holds it and a block's shared memory receives it: the
// block's 32 time steps of every column, in units of 2^E[column].
struct __align__(16) BTile {
    unsigned char B[2][kPlanes][kBPlane];  // [half][part]: K-major BF16, core matrices 8 x 16 B
    int E[kMmaCols];                       // the largest exponent of the column's values (kZeroExp: all zero)
    unsigned char Bsh[kBPlane];            // the hi part of half 1 with column n at (n + 8) mod 16
};
static_assert(sizeof(BTile) == 2 * kPlanes * kBPlane + 64 + kBPlane && sizeof(BTile) % 16 == 0,
              "tiles are whole 16-byte units");
// the bytes a block copies per tile: Bsh only with at most 8 columns in use
constexpr uint32_t kTileBytesShift = (uint32_t)sizeof(BTile);
constexpr uint32_t kTileBytes = (uint32_t)(2 * kPlanes * kBPlane + 64);

struct __align__(128) Smem {
    BTile b[2][2];                  // [buffer][sweep]: block q's tiles in buffer q % 2
    float rescale[3][2][kMmaCols];  // factor for the totals before adding block q's D (slot q % 3)
    float dscale[3][2][kMmaCols];   // factor for block q's D: 2^(its exponent - the running one)
    int grew[3][2];                 // per sweep: some column's running exponent grew at block q
    int ref[2][kMmaCols];           // running exponent per sweep and column
    uint64_t mbar;                  // the MMAs of a block
    uint64_t bbar[2];               // the copies into buffer 0 / 1
    uint32_t tmem;
};

__device__ __forceinline__ float pow2f_or_zero(int d)  // 2^d for d <= 0, 0 below the normal range
{
    return d < -126 ? 0.0f : __int_as_float((d + 127) << 23);
}
// 2^e as a double for e <= 1023, 0 below the normal range (the totals' scales, |e| < 300)
__device__ __forceinline__ double pow2d_or_zero(int e)
{
    return e < -1022 ? 0.0 : __longlong_as_double((long long)(e + 1023) << 52);
}

// Byte offset of element (column n, step k) in a B plane: K-major core matrices,
// 128 B between the two along K (LBO), 256 B between 8-column groups (SBO).
__device__ __forceinline__ int b_off(int n, int k) { return (n >> 3) * 256 + (k >> 3) * 128 + (n & 7) * 16 + (k & 7) * 2; }

__device__ __forceinline__ uint32_t bf2_bits(__nv_bfloat162 v) { return *reinterpret_cast<uint32_t*>(&v); }

// Three-part BF16 split of two values (low half: a, high half: b).
__device__ __forceinline__ void split3(float a, float b, uint32_t (&w)[kPlanes])
{
    const __nv_bfloat162 h = __floats2bfloat162_rn(a, b);
    const float ra = a - __low2float(h), rb = b - __high2float(h);
    const __nv_bfloat162 m = __floats2bfloat162_rn(ra, rb);
    const float qa = ra - __low2float(m), qb = rb - __high2float(m);
    const __nv_bfloat162 l = __floats2bfloat162_rn(qa, qb);
    w[0] = bf2_bits(h);
    w[1] = bf2_bits(m);
    w[2] = bf2_bits(l);
}

// The l3 of time step tau: the (2 -2 0) sweeps move one l3 per step; the (0 0 0) sweeps two,
// from one non-zero point of the family to the next (forward l3 = l2 - l1 + 2 nF, nF = tau - i
// + w - 3; backward l3 = l1 + l2 - 2 nB, nB = tau + w + i - 34).
template <bool F00>
__device__ __forceinline__ int l3_of(int s, int tau, int r0, int c0)
{
    return ps_mma_tiles::l3_at(F00, s, tau, r0, c0);
}
static_assert(ps_mma_tiles::l3_at(false, 0, 0, 0, 0) == -kLead && ps_mma_tiles::l3_at(false, 1, 0, 0, 0) == kRamp,
              "the skew of the (2 -2 0) sweeps");

// ---- the table of B tiles ---------------------------------------------------------
// Entry e < nf is the forward tile of o = fmin + e, entry nf + e the backward tile of o = bmin + e
// (ps_mma_tiles::table_geom: the ranges every block of a launch stays in).
using ps_mma_tiles::TableGeom;
using ps_mma_tiles::table_geom;

// One tile per block of 128 threads: thread = column n (16) x 4 consecutive steps k (8).  The
// (0 0 0) sweeps visit only points where l1 + l2 + l3 is even; a (2 -2 0) slot of one parity
// takes the steps of that parity (l1 + l2 + l3 has the parity of the time step, whose blocks
// start at even steps).  Column nslot is the normalisation, 2 l3 + 1.  With at most 8 columns
// in use, the hi part of half 1 is also written with its columns moved up by 8 (the zero
// columns 8-15 moving down to 0-7), so that its hi x hi product lands in D's spare columns.
template <bool F00>
__global__ void __launch_bounds__(128) k_mma_table(const MmaParams p)
{
    const int e = blockIdx.x, tid = threadIdx.x;
    const int s = e < p.tab_nf ? 0 : 1;
    const int o = s ? p.tab_bmin + (e - p.tab_nf) : p.tab_fmin + e;
    const int n = tid >> 3, kq = tid & 7;
    const int step = F00 ? 2 : 1;
    float m[4];
    int ex[4];
    int emax = kZeroExp;
#pragma unroll
    for (int u = 0; u < 4; ++u) {
        const int k = 4 * kq + u, l3 = s ? o - step * k : o + step * k;
        m[u] = 0.0f;
        ex[u] = kZeroExp;
        if (l3 >= 0 && l3 < p.wlen) {
            if (n < p.nslot) {
                const int par = p.parity[n];
                if (F00 ? par != PAR_ODD : (par == PAR_ALL || (par == PAR_EVEN) == ((k & 1) == 0))) {
                    const int2 v = __ldg(p.bf[n] + l3);
                    m[u] = __int_as_float(v.x);
                    ex[u] = v.y;
                }
            } else if (n == p.nslot) {
                m[u] = frexpf((float)(2 * l3 + 1), &ex[u]);
            }
        }
        emax = max(emax, ex[u]);
    }
    // the column's 8 threads are consecutive lanes
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 1));
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 2));
    emax = max(emax, __shfl_xor_sync(0xffffffffu, emax, 4));
    BTile& T = reinterpret_cast<BTile*>(p.tab)[e];
    if (kq == 0) T.E[n] = emax;
    float v[4];
#pragma unroll
    for (int u = 0; u < 4; ++u) v[u] = m[u] * pow2f_or_zero(ex[u] - emax);
    uint32_t w01[kPlanes], w23[kPlanes];
    split3(v[0], v[1], w01);
    split3(v[2], v[3], w23);
    const int h = kq >> 2, kk = 4 * (kq & 3);
    const int off = b_off(n, kk);
#pragma unroll
    for (int pl = 0; pl < kPlanes; ++pl) *reinterpret_cast<uint2*>(&T.B[h][pl][off]) = make_uint2(w01[pl], w23[pl]);
    if (p.nslot + 1 <= 8 && h == 1)
        *reinterpret_cast<uint2*>(&T.Bsh[b_off((n + 8) & (kMmaCols - 1), kk)]) = make_uint2(w01[0], w23[0]);
}

// One thread starts the copies of block q's two tiles (time steps q kBlk ..) into buffer q % 2.
// An entry outside the table (which the ranges above exclude) is replaced by the first entry of
// its sweep and reported through ok.
template <bool F00>
__device__ __forceinline__ void copy_tiles(const MmaParams& p, Smem& sm, int q, int r0, int c0, uint32_t bytes,
                                           bool& ok)
{
    const int tb = q * kBlk, buf = q & 1;
    umma::mbar_expect_tx(&sm.bbar[buf], 2u * bytes);
#pragma unroll
    for (int s = 0; s < 2; ++s) {
        const int o = l3_of<F00>(s, tb, r0, c0);
        int e = s ? o - p.tab_bmin : o - p.tab_fmin;
        if (e < 0 || e >= (s ? p.tab_nb : p.tab_nf)) {
            ok = false;
            e = 0;
        }
        if (s) e += p.tab_nf;
        umma::bulk_g2s(&sm.b[buf][s], p.tab + (size_t)e * sizeof(BTile), bytes, &sm.bbar[buf]);
    }
}

struct Sweep22 {
    ff f, fo;  // f at the current point and at the previous one
    float w;   // 4 (2 j + 1)
};

// ---- recurrence coefficient rings -------------------------------------------
// For the pair (l1, l2) the recurrence coefficient factorises as
//   forward step t (point j = l2 - l1 + t):  P(j) = G(t) F(v),   v = 2 l2 + t,
//     G(t) = t (2 l1 + 1 - t),  F(v) = (v - 2 l1)(v + 1);
//   backward step t (point j = l1 + l2 - t): P(j) = G(t + 1) Fb(u),  u = 2 l2 - t,
//     Fb(u) = u (2 l1 + 1 + u).
// So rho = a(j)/a(j+1) and r = 1/a(j+1) of a forward step are products of a G
// entry and an F entry,
//   g[t]  = (sqrt(G(t)/G(t+1)), 1/sqrt(G(t+1))),  f[v] = (sqrt(F(v)/F(v+1)), 1/sqrt(F(v+1))),
// and rho = a(j+1)/a(j), r = 1/a(j) of a backward step of g[t] and
//   fb[u] = (sqrt(Fb(u+1)/Fb(u)), 1/sqrt(Fb(u))).
// Each warp (one row l1) keeps the three tables as rings of 64 entries per
// parity.  In the skewed frame t, v and u all have the parity of tau, lane i
// reads entry (index / 2) of consecutive lanes' neighbours (no bank conflicts),
// and the forward and backward sweeps share g (t of the backward sweep of lane
// i is t of the forward sweep of lane 31 - i).  A 32-step block reads 94
// consecutive values of each table (47 per parity); it needs 32 new ones per
// table beyond the block before, built at its start (the ring holds 128).
//
// A block's 16 step pairs read 16 consecutive slots of each table (increasing for g
// and f, decreasing for fb) from a start computed once per block.  So each table
// keeps kGuard slots a second time past its end (g, f: slot s < kGuard also at
// kRing + s) or before its start (fb: slot s at kGuard + s, and slot s >= kRing -
// kGuard also at s - (kRing - kGuard)), and a run of kGuard slots from any start is
// contiguous: no wrap-around arithmetic per step.
constexpr int kRing = 64;
constexpr int kGuard = kBlk / 2;
struct ffpair {
    ff rho, r;
};
struct __align__(16) CoefRing {
    ffpair g[2][kRing + kGuard], f[2][kRing + kGuard], fb[2][kGuard + kRing];
};
__device__ __forceinline__ int ring_slot(int x) { return (x >> 1) & (kRing - 1); }
// store slot s of a table read upwards / downwards in runs of G slots
template <int G, typename T>
__device__ __forceinline__ void put_up(T* t, int s, const T& v)
{
    t[s] = v;
    if (s < G) t[kRing + s] = v;
}
template <int G, typename T>
__device__ __forceinline__ void put_down(T* t, int s, const T& v)
{
    t[G + s] = v;
    if (s >= kRing - G) t[s - (kRing - G)] = v;
}

// (sqrt(X / Y), 1 / sqrt(Y)) of two exact integer products; rho is 0 where X is
__device__ __forceinline__ ffpair ratio_entry(ff X, ff Y)
{
    const ff r = ff_rsqrt(Y);
    const ff rho = X.h > 0.0f ? ff_mul(X, ff_rsqrt(ff_mul_raw(X, Y))) : ff_make(0.0f);
    return ffpair{rho, r};
}
__device__ __forceinline__ void ring_g(CoefRing& R, int t, int l1)
{
    put_up<kGuard>(R.g[t & 1], ring_slot(t),
                   ratio_entry(two_prod((float)t, (float)(2 * l1 + 1 - t)), two_prod((float)(t + 1), (float)(2 * l1 - t))));
}
__device__ __forceinline__ void ring_f(CoefRing& R, int v, int l1)
{
    put_up<kGuard>(R.f[v & 1], ring_slot(v),
                   ratio_entry(two_prod((float)(v - 2 * l1), (float)(v + 1)),
                               two_prod((float)(v + 1 - 2 * l1), (float)(v + 2))));
}
__device__ __forceinline__ void ring_fb(CoefRing& R, int u, int l1)
{
    put_down<kGuard>(R.fb[u & 1], ring_slot(u),
                     ratio_entry(two_prod((float)(u + 1), (float)(2 * l1 + 2 + u)),
                                 two_prod((float)u, (float)(2 * l1 + 1 + u))));
}

// one step of the (2 -2 0) family: f(next) = -(w f r + rho f(prev))
__device__ __forceinline__ void step22(Sweep22& S, ff rho, ff r, float dw)
{
    const ff x = ff_mul_raw(ff_mulf_raw(S.f, S.w), r);
    const ff y = ff_mul_raw(rho, S.fo);
    S.fo = S.f;
    S.f = ff_neg(ff_add_raw(x, y));
    S.w += dw;
}
// Table indices of a lane's first step pair in a block (tau even, then odd): t, v = 2 l2 + t of
// the forward step and t of the backward step are even at the even step, so both steps use the
// same slot of each; u = 2 l2 - t of the backward step is even at the even step and one less at
// the odd one.  Pair k of the block (k < 16) reads g and f at + k and fb at - k.
struct RingIdx {
    int g, f, gb, fb0, fb1;
};
__device__ __forceinline__ RingIdx ring_idx(int tf_even, int tb_even, int l2)
{
    const int u0 = 2 * l2 - tb_even;
    return RingIdx{ring_slot(tf_even), ring_slot(2 * l2 + tf_even), ring_slot(tb_even), kGuard + ring_slot(u0),
                   kGuard + ring_slot(u0 - 1)};
}
// forward step of parity p in pair k: g[t] and f[2 l2 + t]
__device__ __forceinline__ void fwd_step(Sweep22& S, const CoefRing& R, int p, const RingIdx& q, int k)
{
    const ffpair g = R.g[p][q.g + k], f = R.f[p][q.f + k];
    step22(S, ff_mul_raw(g.rho, f.rho), ff_mul_raw(g.r, f.r), 8.0f);
}
// backward step of parity p in pair k: g[t] and fb[2 l2 - t]
__device__ __forceinline__ void bwd_step(Sweep22& S, const CoefRing& R, int p, const RingIdx& q, int k)
{
    const ffpair g = R.g[p][q.gb + k], f = R.fb[p][(p ? q.fb1 : q.fb0) - k];
    step22(S, ff_mul_raw(g.rho, f.rho), ff_mul_raw(g.r, f.r), -8.0f);
}

// ---- the (0 0 0) sweeps --------------------------------------------------------
// The (0 0 0) family vanishes where l1 + l2 + l3 is odd, so its sweeps step two points at a
// time: f(j + 2) = -rho f(j) with rho the product of the odd-t entries of the (2 -2 0) step
// (forward g[t] f[2 l2 + t], backward g[t] fb[2 l2 - t], t = 2n + 1 at step n), whose rho alone
// is needed.  Each warp keeps them as rings of 64 odd values; a 32-step block reads 63
// consecutive ones of each table, 32 of them new, built at its start.
constexpr int kGuard00 = kBlk;  // a block's 32 steps read 32 consecutive slots of each table
struct __align__(16) Ring00 {
    ff g[kRing + kGuard00], f[kRing + kGuard00], fb[kGuard00 + kRing];  // slot (x >> 1) & 63 of odd x
};
// sqrt(X / Y) of two exact integer products, 0 where X is
__device__ __forceinline__ ff rho_entry(ff X, ff Y)
{
    return X.h > 0.0f ? ff_mul(X, ff_rsqrt(ff_mul_raw(X, Y))) : ff_make(0.0f);
}
// the odd values of the block starting at time step tb: t in [tlo, tlo + 124], v in
// [vlo, vlo + 124], u in [ulo, ulo + 124]
__device__ __forceinline__ int ring00_tlo(int tb, int w) { return 2 * tb + 2 * w - 67; }
__device__ __forceinline__ int ring00_vlo(int tb, int w, int c0) { return 2 * c0 + 2 * w + 2 * tb - 5; }
__device__ __forceinline__ int ring00_ulo(int tb, int w, int c0) { return 2 * c0 - 2 * w + 5 - 2 * tb; }
// One entry of g (isf false) or f (isf true) at odd x: P(x) = a0 b0, P(x + 1) = (a0 + 1)(b0 -+ 1)
__device__ __forceinline__ void ring00_gf(Ring00& R, int x, bool isf, int l1)
{
    const float a0 = (float)(isf ? x - 2 * l1 : x), b0 = (float)(isf ? x + 1 : 2 * l1 + 1 - x);
    const ff rho = rho_entry(two_prod(a0, b0), two_prod(a0 + 1.0f, isf ? b0 + 1.0f : b0 - 1.0f));
    put_up<kGuard00>(isf ? R.f : R.g, ring_slot(x), rho);
}
// One entry of fb at odd u: sqrt(Fb(u + 1) / Fb(u)), Fb(u) = u (2 l1 + 1 + u)
__device__ __forceinline__ void ring00_fb(Ring00& R, int u, int l1)
{
    const float a0 = (float)u, b0 = (float)(2 * l1 + 1 + u);
    put_down<kGuard00>(R.fb, ring_slot(u), rho_entry(two_prod(a0 + 1.0f, b0 + 1.0f), two_prod(a0, b0)));
}
__device__ __forceinline__ void build_rings00_first(Ring00& R, int tb, int w, int l1, int c0, int lane)
{
    const int tlo = ring00_tlo(tb, w), vlo = ring00_vlo(tb, w, c0), ulo = ring00_ulo(tb, w, c0);
    for (int e = lane; e < 63; e += 32) {
        ring00_gf(R, tlo + 2 * e, false, l1);
        ring00_gf(R, vlo + 2 * e, true, l1);
        ring00_fb(R, ulo + 2 * e, l1);
    }
}
// The 32 values per table that block tb needs beyond the block before: the top 32 of t and v,
// the bottom 32 of u, one per lane in each of three passes.
__device__ __forceinline__ void build_rings00_next(Ring00& R, int tb, int w, int l1, int c0, int lane)
{
    ring00_gf(R, ring00_tlo(tb, w) + 62 + 2 * lane, false, l1);
    ring00_gf(R, ring00_vlo(tb, w, c0) + 62 + 2 * lane, true, l1);
    ring00_fb(R, ring00_ulo(tb, w, c0) + 2 * lane, l1);
}
// Table indices of a lane's first step in a block: forward step n reads g at t = 2n + 1 (slot
// n) and f at v = 2 l2 + t (slot l2 + n); backward step n reads g at t (slot n) and fb at
// u = 2 l2 - t (slot l2 - n - 1).  Step j of the block reads g and f at + j and fb at - j.
struct RingIdx00 {
    int g, f, gb, fb;
};
__device__ __forceinline__ RingIdx00 ring00_idx(int nf, int nb, int l2)
{
    return RingIdx00{nf & (kRing - 1), (l2 + nf) & (kRing - 1), nb & (kRing - 1),
                     kGuard00 + ((l2 - nb - 1) & (kRing - 1))};
}
__device__ __forceinline__ void fwd_step00c(ff& f, const Ring00& R, const RingIdx00& q, int j)
{
    f = ff_neg(ff_mul_raw(ff_mul_raw(R.g[q.g + j], R.f[q.f + j]), f));
}
__device__ __forceinline__ void bwd_step00c(ff& f, const Ring00& R, const RingIdx00& q, int j)
{
    f = ff_neg(ff_mul_raw(ff_mul_raw(R.g[q.gb + j], R.fb[q.fb - j]), f));
}

// sqrt(X / Y) for the last forward points (X, Y up to 2^64: the scaling keeps X Y in range)
__device__ __forceinline__ ff rho00(ff X, ff Y)
{
    const ff Xs = ff{X.h * 0x1p-32f, X.l * 0x1p-32f};
    const ff r = ff_mul(Xs, ff_rsqrt(ff_mul_raw(Xs, Y)));
    return ff{r.h * 0x1p16f, r.l * 0x1p16f};
}

// The ring values of the block starting at time step tb, for warp row l1 = r0 + 2w and lanes
// l2 = c0 + 2i: t in [tlo, tlo + 93], v in [vlo, vlo + 93], u in [ulo, ulo + 93].
__device__ __forceinline__ int ring_tlo(int tb, int w) { return tb - 68 + 2 * w; }
__device__ __forceinline__ int ring_vlo(int tb, int w, int c0) { return 2 * c0 + 2 * w + tb - 6; }
__device__ __forceinline__ int ring_ulo(int tb, int w, int c0) { return 2 * c0 - 2 * w + 37 - tb; }

// All 94 values of each table (the first block).
__device__ __forceinline__ void build_rings_first(CoefRing& R, int tb, int w, int l1, int c0, int lane)
{
    const int tlo = ring_tlo(tb, w), vlo = ring_vlo(tb, w, c0), ulo = ring_ulo(tb, w, c0);
    for (int e = lane; e < 94; e += 32) {
        ring_g(R, tlo + e, l1);
        ring_f(R, vlo + e, l1);
        ring_fb(R, ulo + e, l1);
    }
}

// The 32 values per table that block tb needs beyond the block before: the top 32 of t and v,
// the bottom 32 of u.  With s(x) = 1/sqrt(P(x)) for the table's products P,
//   g, f entry x  = (sqrt(P(x) / P(x+1)), 1/sqrt(P(x+1))) = (P(x) s(x) s(x+1), s(x+1)),
//   fb entry x    = (sqrt(P(x+1) / P(x)), 1/sqrt(P(x)))   = (P(x+1) s(x+1) s(x), s(x)),
// so a new entry takes one float-float 1/sqrt; the neighbouring s comes from the next lane or,
// at the edge of the 32, from the entry of the block before that holds it as its r.  P(x) is 0
// only at the first step of a sweep, where the entry's rho is 0.  One pass per table, one
// entry per lane.
__device__ __forceinline__ void ring_gf_next(CoefRing& R, int x, bool isf, int l1, int lane)
{
    // g: P(x) = x (2 l1 + 1 - x), P(x + 1) = (x + 1)(2 l1 - x)
    // f: P(x) = (x - 2 l1)(x + 1), P(x + 1) = (x + 1 - 2 l1)(x + 2)
    const float a0 = (float)(isf ? x - 2 * l1 : x), b0 = (float)(isf ? x + 1 : 2 * l1 + 1 - x);
    const ff s1 = ff_rsqrt(two_prod(a0 + 1.0f, isf ? b0 + 1.0f : b0 - 1.0f));
    ff s0{__shfl_up_sync(0xffffffffu, s1.h, 1), __shfl_up_sync(0xffffffffu, s1.l, 1)};
    ffpair(*tab)[kRing + kGuard] = isf ? R.f : R.g;
    if (lane == 0) s0 = tab[(x - 1) & 1][ring_slot(x - 1)].r;
    const ff P0 = two_prod(a0, b0);
    const ff rho = P0.h > 0.0f ? ff_mul(ff_mul_raw(P0, s0), s1) : ff_make(0.0f);
    put_up<kGuard>(tab[x & 1], ring_slot(x), ffpair{rho, s1});
}
__device__ __forceinline__ void build_rings_next(CoefRing& R, int tb, int w, int l1, int c0, int lane)
{
    ring_gf_next(R, ring_tlo(tb, w) + 62 + lane, false, l1, lane);
    ring_gf_next(R, ring_vlo(tb, w, c0) + 62 + lane, true, l1, lane);
    const int x = ring_ulo(tb, w, c0) + lane;  // Fb(x) = x (2 l1 + 1 + x)
    const float a0 = (float)x, b0 = (float)(2 * l1 + 1 + x);
    const ff s0 = ff_rsqrt(two_prod(a0, b0));
    ff s1{__shfl_down_sync(0xffffffffu, s0.h, 1), __shfl_down_sync(0xffffffffu, s0.l, 1)};
    if (lane == 31) s1 = R.fb[(x + 1) & 1][kGuard + ring_slot(x + 1)].r;
    const ff P1 = two_prod(a0 + 1.0f, b0 + 1.0f);
    const ff rho = P1.h > 0.0f ? ff_mul(ff_mul_raw(P1, s1), s0) : ff_make(0.0f);
    put_down<kGuard>(R.fb[x & 1], ring_slot(x), ffpair{rho, s0});
}

__device__ __forceinline__ float sq(const ff& f)
{
    const float g = __fadd_rn(f.h, f.l);
    return __fmul_rn(g, g);
}

// The totals take each block's D into their low word (one FP32 add), and the columns
// n = R (mod 4) are renormalised by a two-sum at blocks q = R (mod 4).  So a low word sums at
// most four blocks between renormalisations: at most four roundings of 2^-24 relative to those
// blocks' sum, against one rounding of the tensor core's truncating accumulation per block.
template <int R, int NC>
__device__ __forceinline__ void renorm(ff (&t)[NC], int ncols)
{
#pragma unroll
    for (int n = R; n < NC; n += 4)
        if (n < ncols) t[n] = two_sum(t[n].h, t[n].l);
}

template <bool F00>
using RingT = typename std::conditional<F00, Ring00, CoefRing>::type;

// NC: columns folded into the totals (8 or 16; at least nslot + 1).  STAGE: the outputs are
// in host memory (MmaParams::stage_rows).
template <bool F00, int NC, bool STAGE>
__global__ void __launch_bounds__(128) k_coupling_mma(const MmaParams p)
{
    __shared__ Smem sm;
    extern __shared__ __align__(16) unsigned char dyn[];  // the warps' coefficient rings
    const int tid = threadIdx.x, warp = tid >> 5, lane = tid & 31;
    RingT<F00>& R = reinterpret_cast<RingT<F00>*>(dyn)[warp];
    const int2 tile = p.tiles[blockIdx.x];
    const int r0 = tile.x, c0 = tile.y;
    const int l1 = r0 + 2 * warp, l2 = c0 + 2 * lane;
    const bool writes = l1 >= p.lmin && l1 <= p.lmax && l2 >= l1 && l2 <= p.lmax;
    const bool runs = writes && (F00 || l1 >= 2);  // the (2 -2 0) family vanishes for l1 < 2
    const int T = runs ? l1 : 0;
    const int d = l2 - l1;
    // block q covers the time steps q kBlk .. q kBlk + 31; the sweeps run for tau in
    // [0, r0 + kRamp) ((2 -2 0)) or [0, floor((r0 + 1) / 2) + 34) ((0 0 0), two points per step)
    const int ntau = ps_mma_tiles::nsteps(F00, r0);
    const int nk = (ntau + kBlk - 1) / kBlk;  // 32-step blocks of the skewed sweeps (block-uniform)
    const int ncols = p.nslot + 1;
    // With at most 8 columns (NC == 8) D's columns 8-15 are spare: the hi x hi product of the
    // block's second half goes there on its own (its B columns moved up by 8), and the fold adds
    // the two column halves.  Each hi x hi product then takes its rounding toward zero at the
    // scale of its own 16 steps, as with one D per 16 steps.
    constexpr bool kShift = NC == 8;

    constexpr uint32_t kBytes = kShift ? kTileBytesShift : kTileBytes;
    bool ok = true;

    if (warp == 0) umma::tmem_alloc(&sm.tmem, kTmemCols);
    if (tid < 2 * kMmaCols) sm.ref[tid / kMmaCols][tid % kMmaCols] = kZeroExp;
    if (tid == 0) {
        umma::mbar_init(&sm.mbar, 2);  // one commit per sweep
        umma::mbar_init(&sm.bbar[0]);
        umma::mbar_init(&sm.bbar[1]);
    }
    umma::fence_before_sync();
    __syncthreads();
    umma::fence_after_sync();
    const uint32_t tbase = sm.tmem;
    const uint32_t tlane = tbase + ((uint32_t)(32 * warp) << 16);
    const uint64_t bdesc0 = umma::smem_desc(umma::smem_addr(&sm.b[0][0]), 128u, 256u);  // B[0] of buffer 0, sweep 0
    if (tid == 0) {  // the tiles of blocks 0 and 1 (both buffers are free)
        copy_tiles<F00>(p, sm, 0, r0, c0, kBytes, ok);
        if (nk > 1) copy_tiles<F00>(p, sm, 1, r0, c0, kBytes, ok);
    }
    if constexpr (F00) build_rings00_first(R, 0, warp, l1, c0, lane);
    else build_rings_first(R, 0, warp, l1, c0, lane);

    // sweep state: the (2 -2 0) family with its recurrence coefficient, or (f alone) the (0 0 0) family
    Sweep22 F, B;
    F.f = ff_make(1.0f); F.fo = ff_make(0.0f); F.w = 4.0f * (float)(2 * d + 1);
    B.f = ff_make(1.0f); B.fo = ff_make(0.0f); B.w = 4.0f * (float)(2 * (l1 + l2) + 1);
    ff tot[2][NC];
#pragma unroll
    for (int s = 0; s < 2; ++s)
#pragma unroll
        for (int n = 0; n < NC; ++n) tot[s][n] = ff_make(0.0f);

    // The last warp, lane = sweep (lane / 16) x column (lane % 16), once block q's tiles have
    // arrived: the column's running exponent (in a register and in sm.ref) and the factors that
    // the fold of block q applies, to the totals where the running exponent grows and to D.
    // (The first warp starts the copies, the first two issue the MMAs.)
    int ref = kZeroExp;
    auto scales = [&](int q) {
        const int s = lane >> 4, n = lane & (kMmaCols - 1);
        ok &= umma::mbar_wait(&sm.bbar[q & 1], (uint32_t)((q >> 1) & 1), kWaitLimit);
        const int E = sm.b[q & 1][s].E[n];
        float dsc = 0.0f, rsc = 1.0f;
        bool grew = false;
        if (E != kZeroExp) {
            if (E > ref) {
                rsc = pow2f_or_zero(ref - E);
                dsc = 1.0f;
                ref = E;
                sm.ref[s][n] = E;
                grew = true;
            } else {
                dsc = pow2f_or_zero(E - ref);
            }
        }
        sm.dscale[q % 3][s][n] = dsc;
        sm.rescale[q % 3][s][n] = rsc;
        const unsigned g = __ballot_sync(0xffffffffu, grew);
        if (lane == 0) {
            sm.grew[q % 3][0] = (g & 0xffffu) != 0u;
            sm.grew[q % 3][1] = (g >> 16) != 0u;
        }
    };

    auto flush = [&](int q) {
        ok &= umma::mbar_wait(&sm.mbar, (uint32_t)(q & 1), kWaitLimit);
        __syncwarp();  // lanes leave the wait at different polls; the loads below are warp-collective
        umma::fence_after_sync();
#pragma unroll
        for (int s = 0; s < 2; ++s) {
            float dv[kMmaCols];
            umma::ld_x16(tlane + (uint32_t)(s * kMmaCols), dv);
            // the totals move to the new running exponent where it grew (the same for every
            // thread: a uniform branch, taken only when some window's exponent grew)
            if (sm.grew[q % 3][s]) {
                const float4* rs = reinterpret_cast<const float4*>(&sm.rescale[q % 3][s][0]);
#pragma unroll
                for (int v = 0; v < NC / 4; ++v) {
                    const float4 r4 = rs[v];
                    const float rv[4] = {r4.x, r4.y, r4.z, r4.w};
#pragma unroll
                    for (int j = 0; j < 4; ++j) {
                        tot[s][4 * v + j].h *= rv[j];
                        tot[s][4 * v + j].l *= rv[j];
                    }
                }
            }
            if (kShift) {
#pragma unroll
                for (int n = 0; n < NC; ++n) dv[n] = __fadd_rn(dv[n], dv[n + 8]);
            }
            // D in units of 2^(block exponent), brought to the running exponent (an exact power of two)
            const float4* ds = reinterpret_cast<const float4*>(&sm.dscale[q % 3][s][0]);
#pragma unroll
            for (int v = 0; v < NC / 4; ++v) {
                const float4 d4 = ds[v];
                const float dw[4] = {d4.x, d4.y, d4.z, d4.w};
#pragma unroll
                for (int j = 0; j < 4; ++j)
                    if (4 * v + j < ncols) tot[s][4 * v + j].l = __fmaf_rn(dv[4 * v + j], dw[j], tot[s][4 * v + j].l);
            }
            switch (q & 3) {
                case 0: renorm<0>(tot[s], ncols); break;
                case 1: renorm<1>(tot[s], ncols); break;
                case 2: renorm<2>(tot[s], ncols); break;
                default: renorm<3>(tot[s], ncols); break;
            }
        }
    };

    // (2 -2 0): forward step tF = tau + fofs, backward tB = tau + bofs (one point each);
    // (0 0 0): forward step nF = tau + fofs, backward nB = tau + bofs (two points each)
    const int fofs = F00 ? warp - lane - 3 : -kLead - 2 * lane + 2 * warp;
    const int bofs = F00 ? warp + lane - 34 : 2 * warp + 2 * lane - kRamp;
    // (0 0 0): both sweeps take (T + 1) / 2 points; the forward one steps after each (ending at
    // l2 or l2 + 1), the backward one after all but the last when T is odd (ending there too).
    // From tau = 34 to floor((r0 + 1) / 2) + 1 every lane that runs is inside both sweeps.
    const int nx00 = (T + 1) / 2, ns00 = T / 2, steady00 = ((r0 + 1) >> 1) + 1;
    for (int q = 0; q < nk; ++q) {
        const int tb = q * kBlk;  // the block's first time step
        // ---- block start: the A operand and D are single-buffered, B double-buffered ----
        if (q > 0) {
            // the ring values of this block (no MMA reads them), then the MMAs of block q - 1
            // (issued at its end): D into the totals; A and the B buffer of q - 1 may be
            // overwritten after, the latter by block q + 1's tiles
            if constexpr (F00) build_rings00_next(R, tb, warp, l1, c0, lane);
            else build_rings_next(R, tb, warp, l1, c0, lane);
            flush(q - 1);
            if (tid == 0 && q + 1 < nk) copy_tiles<F00>(p, sm, q + 1, r0, c0, kBytes, ok);
        }
        if (warp == 3) scales(q);
        __syncwarp();  // the ring values of the block, written by the warp's lanes
        // the ring indices of the block's first time step (first step pair)
        RingIdx00 ix00;
        RingIdx ix22;
        if constexpr (F00) ix00 = ring00_idx(tb + fofs, tb + bofs, l2);
        else ix22 = ring_idx(tb + fofs, tb + bofs, l2);
        // One step pair of the block: the steps of both sweeps, and x of both as split words.  In
        // a block whose steps all lie in the steady state, every lane that runs is inside both
        // sweeps, so both steps run unconditionally (their dependency chains interleave).  Lanes
        // that do not run compute values that may not be finite: they reach only their own rows
        // of the MMAs (row m of D is row m of A times B) and their own totals, never written.
        // The other blocks (the first few and the last) check every step.
        auto pair = [&](int s2, bool steady, uint32_t (&wf)[kPlanes], uint32_t (&wb)[kPlanes]) {
            float xf[2], xb[2];
            const int tau0 = tb + s2;
            if constexpr (F00) {
#pragma unroll
                for (int e = 0; e < 2; ++e) {
                    const int nf = tau0 + e + fofs, nb = tau0 + e + bofs;
                    if (steady) {
                        xf[e] = sq(F.f);
                        xb[e] = sq(B.f);
                        fwd_step00c(F.f, R, ix00, s2 + e);
                        bwd_step00c(B.f, R, ix00, s2 + e);
                    } else {
                        xf[e] = 0.0f;
                        xb[e] = 0.0f;
                        if (nf >= 0 && nf < nx00) {
                            xf[e] = sq(F.f);
                            fwd_step00c(F.f, R, ix00, s2 + e);
                        }
                        if (nb >= 0 && nb < nx00) {
                            xb[e] = sq(B.f);
                            if (nb < ns00) bwd_step00c(B.f, R, ix00, s2 + e);
                        }
                    }
                }
            } else {
                const int k = s2 >> 1;  // the step pair of the block
#pragma unroll
                for (int e = 0; e < 2; ++e) {  // e: the step parity (tau even, then odd)
                    const int tf = tau0 + e + fofs, tbk = tau0 + e + bofs;
                    if (steady) {
                        xf[e] = sq(F.f);
                        xb[e] = sq(B.f);
                        fwd_step(F, R, e, ix22, k);
                        bwd_step(B, R, e, ix22, k);
                    } else {
                        xf[e] = 0.0f;
                        xb[e] = 0.0f;
                        if (tf >= 0 && tf < T) {
                            xf[e] = sq(F.f);
                            fwd_step(F, R, e, ix22, k);
                        }
                        if (tbk >= 0 && tbk < T) {
                            xb[e] = sq(B.f);
                            bwd_step(B, R, e, ix22, k);
                        }
                    }
                }
            }
            split3(xf[0], xf[1], wf);
            split3(xb[0], xb[1], wb);
        };
        // Two step pairs (s2 .. s2 + 3), then their x into tensor memory: step pairs k and k + 1
        // of the block in two consecutive columns of each sweep and plane, one store each.
        auto two_pairs = [&](int s2, bool steady) {
            uint32_t wf0[kPlanes], wb0[kPlanes], wf1[kPlanes], wb1[kPlanes];
            pair(s2, steady, wf0, wb0);
            pair(s2 + 2, steady, wf1, wb1);
            __syncwarp();  // the stores below are warp-collective (.sync.aligned)
            const uint32_t k = (uint32_t)(s2 >> 1);  // the first step pair
#pragma unroll
            for (int pl = 0; pl < kPlanes; ++pl) {
                umma::st_x2(tlane + a_col(0, pl) + k, wf0[pl], wf1[pl]);
                umma::st_x2(tlane + a_col(1, pl) + k, wb0[pl], wb1[pl]);
            }
        };
        const int t1 = tb + kBlk - 1;  // the block's last time step
        const bool steady = F00 ? (tb >= 34 && t1 <= steady00) : (tb >= kSteady && t1 <= r0 + kLead - 1);
        if (steady) {
#pragma unroll 1
            for (int s2 = 0; s2 < kBlk; s2 += 4) two_pairs(s2, true);
        } else {
#pragma unroll 1
            for (int s2 = 0; s2 < kBlk; s2 += 4) two_pairs(s2, false);
        }
        // ---- block end: A complete; lane 0 of warp s issues sweep s's 12 MMAs once it has seen
        // the block's tiles arrive, and commits them (the barrier's phase needs both commits) ----
        umma::wait_st();
        umma::fence_before_sync();
        __syncthreads();
        umma::fence_after_sync();
        // the five small products of both halves first, hi x hi of both last; the first MMA
        // starts D from zero.  Descriptors of buffer q % 2: the first one's plus the planes'
        // offsets (in 16-byte units, within the 14-bit address field: shared memory lies below
        // 256 KB)
        auto issue = [&](auto sweep) {
            constexpr int s = decltype(sweep)::value;
            ok &= umma::mbar_wait(&sm.bbar[q & 1], (uint32_t)((q >> 1) & 1), kWaitLimit);
            const uint64_t bq = bdesc0 + (uint64_t)((q & 1) * (2 * sizeof(BTile) / 16) + s * (sizeof(BTile) / 16));
#pragma unroll
            for (int ps = 0; ps < 6; ++ps)
#pragma unroll
                for (int h = 0; h < 2; ++h) {
                    const uint32_t off = kShift && ps == 5 && h == 1 ? (uint32_t)offsetof(BTile, Bsh)
                                                                     : (uint32_t)((h * kPlanes + kPass[ps][1]) * kBPlane);
                    umma::mma_bf16_ts(tbase + (uint32_t)(s * kMmaCols), tbase + a_col(s, kPass[ps][0], h),
                                      bq + (off >> 4), kIdesc, ps > 0 || h > 0);
                }
            umma::mma_commit(&sm.mbar);
        };
        if (tid == 0) issue(std::integral_constant<int, 0>{});
        else if (tid == 32) issue(std::integral_constant<int, 1>{});
    }
    flush(nk - 1);
    if (!ok) atomicExch(p.status, 1u);

    // ---- the last forward point, match, normalisation (FP64) ----
    double Xi[kMmaMaxSlots];
#pragma unroll
    for (int k = 0; k < kMmaMaxSlots; ++k) Xi[k] = 0.0;
    if (runs) {
        double FW[NC], BW[NC];
#pragma unroll
        for (int n = 0; n < NC; ++n) {
            FW[n] = BW[n] = 0.0;
            if (n < ncols) {
                FW[n] = ((double)tot[0][n].h + (double)tot[0][n].l) * pow2d_or_zero(sm.ref[0][n]);
                BW[n] = ((double)tot[1][n].h + (double)tot[1][n].l) * pow2d_or_zero(sm.ref[1][n]);
            }
        }
        const int jm = l2;  // jmin + T: the last forward point, in FP64; its parity is that of T
        const bool evenT = (T & 1) == 0;
        double gm0, lam;
        double x = 0.0;
        if (F00) {
            // both sweeps end at jm when T is even (a point neither summed) and at jm + 1
            // otherwise (summed by the backward sweep; jm is a zero of the family) and are
            // matched there
            gm0 = ff_to_double(F.f);
            if (evenT) x = gm0 * gm0;
            lam = gm0 / ff_to_double(B.f);
        } else {
            gm0 = ff_to_double(F.f);
            x = gm0 * gm0;
            // one more forward step for f(jm + 1): P(jm) = T(2d+T)(2l1+1-T)(2l2+T+1),
            // P(jm + 1) = (T+1)(2d+T+1)(2l1-T)(2l2+T+2)
            const ff P0 = ff_mul_raw(two_prod((float)T, (float)(2 * d + T)),
                                     two_prod((float)(2 * l1 + 1 - T), (float)(2 * l2 + T + 1)));
            const ff P1 = ff_mul_raw(two_prod((float)(T + 1), (float)(2 * d + T + 1)),
                                     two_prod((float)(2 * l1 - T), (float)(2 * l2 + T + 2)));
            const ff r = ff_rsqrt(P1);
            const double gm1 =
                ff_to_double(ff_neg(ff_add(ff_mul_raw(ff_mulf_raw(F.f, F.w), r), ff_mul_raw(rho00(P0, P1), F.fo))));
            const double hm0 = ff_to_double(B.f), hm1 = ff_to_double(B.fo);
            lam = (gm0 * hm0 + gm1 * hm1) / (hm0 * hm0 + hm1 * hm1);
        }
        const double FN = FW[p.nslot] + (2.0 * jm + 1.0) * x;
        const double BN = BW[p.nslot];
#pragma unroll
        for (int k = 0; k < NC - 1; ++k) {
            if (k < p.nslot) {
                const int par = p.parity[k];
                if (par == PAR_ALL || (par == PAR_EVEN) == evenT) FW[k] = fma(x, __ldg(p.wW[k] + jm), FW[k]);
            }
        }
        const double lam2 = lam * lam;
        const double inv = kInv4Pi / fma(lam2, BN, FN);
#pragma unroll
        for (int k = 0; k < NC - 1; ++k)
            if (k < p.nslot) Xi[k] = fma(lam2, BW[k], FW[k]) * inv;
    }
    // Outputs (column-major, element (row, col) at row + col ldo).  M[l2, l1], the column l1 of
    // the warp's row, is written directly: its lanes' rows step by 2, 16 bytes apart.  M[l1, l2]
    // puts each lane in a different column: written directly to device memory (L2 merges the
    // words), but for outputs in host memory, where each such store crosses NVLink-C2C on its
    // own, it goes through shared memory (the rings' space: every warp has passed its last step)
    // and each warp writes 8 columns with the block's 4 rows of each in one store instruction,
    // 4 words within 64 bytes of a column.
    const bool mcm = p.epilogue == EPI_MCM;
    double* so = reinterpret_cast<double*>(dyn);  // [slot][w][i]
    if (writes) {
        const long long ra = l1 - p.lmin, rb = l2 - p.lmin;
#pragma unroll
        for (int k = 0; k < kMmaMaxSlots; ++k) {
            if (k < p.nslot) {
                const double row = mcm ? (2.0 * l2 + 1.0) * Xi[k] : Xi[k];
                if (STAGE) so[(k * 4 + warp) * 32 + lane] = row;
                else p.out[k][ra + rb * p.ldo] = row;
                p.out[k][rb + ra * p.ldo] = mcm ? (2.0 * l1 + 1.0) * Xi[k] : Xi[k];
            }
        }
    }
    if (STAGE) {
        __syncthreads();
        const int v = lane & 3, i = 8 * warp + (lane >> 2);  // row r0 + 2v, column c0 + 2i
        const int l1v = r0 + 2 * v, l2i = c0 + 2 * i;
        if (l1v >= p.lmin && l1v <= p.lmax && l2i >= l1v && l2i <= p.lmax) {
            const long long off = (l1v - p.lmin) + (long long)(l2i - p.lmin) * p.ldo;
#pragma unroll
            for (int k = 0; k < kMmaMaxSlots; ++k)
                if (k < p.nslot) p.out[k][off] = so[(k * 4 + v) * 32 + i];
        }
    }
    umma::fence_before_sync();
    __syncthreads();
    if (warp == 0) umma::tmem_free(tbase, kTmemCols);
}

// Shared memory per block: the static Smem plus the four warps' coefficient rings
// (dynamic), padded to the 48 KB a block may take without opting in.  That caps
// residency at four blocks per SM, so the four blocks' tensor memory (4 x 128
// columns) fits the SM's 512 columns: no allocation has to wait.
constexpr int kBlockSmem = 48 * 1024;
constexpr int kOccupancySmem = kBlockSmem - (int)sizeof(Smem);
static_assert(4 * sizeof(CoefRing) <= kOccupancySmem, "the rings fit the block's dynamic shared memory");
static_assert(kMmaMaxSlots * 128 * sizeof(double) <= kOccupancySmem, "the staged row halves fit the dynamic shared memory");
static_assert(5 * (kBlockSmem + 1024) > 228 * 1024 && 4 * (kBlockSmem + 1024) <= 228 * 1024,
              "four blocks per SM (1 KB reserved per block)");

}  // namespace

// The blocks of one grid: rows r0 + 2w (w = 0..3) by columns c0 + 2i (i = 0..31),
// in four classes of (row parity, column parity), heaviest (largest r0) first.
void mma_tile_list(int lmin, int lmax, std::vector<int2>& t)
{
    std::vector<std::pair<int, int>> b;
    ps_mma_tiles::block_list(lmin, lmax, b);
    t.resize(b.size());
    for (size_t i = 0; i < b.size(); ++i) t[i] = make_int2(b[i].first, b[i].second);
}

size_t mma_table_bytes(int lmax)
{
    const TableGeom g = table_geom(lmax < 0 ? 0 : lmax);
    return (size_t)(g.nf + g.nb) * sizeof(BTile);
}

cudaError_t launch_mma(const MmaParams& p0, bool fam00, cudaStream_t s)
{
    if (p0.ntiles <= 0) return cudaSuccess;
    if (!p0.tab || ((uintptr_t)p0.tab & 15u) || p0.lmax < 0) return cudaErrorInvalidValue;
    static_assert(sizeof(Smem) + kOccupancySmem <= 48 * 1024, "within the default shared memory limit");
    MmaParams p = p0;
    const TableGeom g = table_geom(p.lmax);
    p.tab_fmin = g.fmin;
    p.tab_nf = g.nf;
    p.tab_bmin = g.bmin;
    p.tab_nb = g.nb;
    if (fam00) k_mma_table<true><<<(unsigned)(g.nf + g.nb), 128, 0, s>>>(p);
    else k_mma_table<false><<<(unsigned)(g.nf + g.nb), 128, 0, s>>>(p);
    if (cudaError_t e = cudaGetLastError()) return e;
    const unsigned grid = (unsigned)p.ntiles;
    auto go = [&](auto kernel) { kernel<<<grid, 128, kOccupancySmem, s>>>(p); };
    const bool nc8 = p.nslot + 1 <= 8, stage = p.stage_rows != 0;
    if (fam00) {
        if (nc8) stage ? go(k_coupling_mma<true, 8, true>) : go(k_coupling_mma<true, 8, false>);
        else stage ? go(k_coupling_mma<true, 16, true>) : go(k_coupling_mma<true, 16, false>);
    } else {
        if (nc8) stage ? go(k_coupling_mma<false, 8, true>) : go(k_coupling_mma<false, 8, false>);
        else stage ? go(k_coupling_mma<false, 16, true>) : go(k_coupling_mma<false, 16, false>);
    }
    return cudaGetLastError();
}

}  // namespace ps
