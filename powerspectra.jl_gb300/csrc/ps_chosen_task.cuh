// ps_chosen_task.cuh -- the chosen coupling kernel's warp task, shared by the
// translation units that instantiate it (ps_chosen.cu, ps_chosen8.cu,
// ps_batch_chosen.cu): FP32-pipe recurrences with
// two-word compensation, block-floating-point windows, FP64 anchors.
//
// Same work and mapping as the plain kernel (one warp = 32 consecutive l2 of one
// l1 row; families (l1 l2 l3; 0 0 0) and (l1 l2 l3; -2 2 0) in registers,
// contracted on the fly; see ps_plain_fp64.cu for the recurrence), with the
// arithmetic moved off the FP64 pipe:
//
//  * recurrence state and coefficients are float-float values (ps_ff.cuh), so
//    each step carries ~2^-46 relative error instead of FP32's 2^-24.  The
//    step factors a(j)/a(j+1) and 1/a(j+1) split into a lane-uniform part and
//    a part shared along u = 2i + t (see "coefficient tables" below); each
//    chunk the warp tabulates both as float-float square-root ratios formed
//    from exact integer products (FP32 1/sqrt estimate plus one compensated
//    Newton step), and every step multiplies two table entries;
//  * the forward (from jmin) and backward (from jmax) sweeps run interleaved
//    in one loop: two independent dependency chains per lane;
//  * windows are stored as (mantissa, exponent) pairs.  Every 32 steps each
//    warp stages the slice of every window it is about to read into shared
//    memory, scaled by 2^-E with E the largest exponent of the slice, so FP32
//    keeps full relative precision whatever the windows' dynamic range
//    (mask spectra span > 1e-45 at l ~ 8000).  The 32-step FP32 partial sums
//    are added into FP64 totals with the factor 2^E;
//  * FP64 is kept where stability and range need it: the last forward point,
//    the least-squares match of the two sweeps, the normalisation, the sign and
//    the totals;
//  * the launch-per-call kernel (k_coupling_chosen) takes a tiled task list:
//    the four warps of a block hold four consecutive rows over one 32-column
//    block, and write the row halves of their pairs together as 32-byte runs
//    (write_tile in ps_epilogue.cuh).  The persistent batch kernel writes per
//    warp (chosen_task).
#pragma once

#include "ps_internal.cuh"
#include "ps_epilogue.cuh"
#include "ps_ff.cuh"

#include <stdint.h>

namespace ps {

constexpr int kChunk = 32;               // steps between window restaging / FP64 flushes
constexpr int kSlots = kChunk + 32;      // staged window entries per warp, direction and window
constexpr int kStagePerLane = kSlots / 32;

__device__ __forceinline__ double pow2d(int e)
{
    e = e < -1022 ? -1022 : (e > 1023 ? 1023 : e);
    return __longlong_as_double((long long)(e + 1023) << 52);
}

__device__ __forceinline__ float pow2f_or_zero(int d)  // 2^d for d <= 0, 0 below the normal range
{
    return d < -126 ? 0.0f : __int_as_float((d + 127) << 23);
}

// A running sum of FP32 chunk partials c 2^e (e: the slice exponent of the
// chunk, the same for every lane of the warp).  ChunkSum<false> adds them into
// FP64 (a conversion and a DFMA per add); ChunkSum<true> keeps the sum on the
// FP32 pipe as a float-float value relative to a running power of two R: when
// a chunk's exponent exceeds R the value is rescaled by 2^(R - e) (exact) and R
// moves up, then c 2^(e - R) is added with Knuth's two-sum.  On GB300 the FP64
// pipe is a small fraction of the FP32 one, and kernels that flush many
// windows per chunk were bound by it.
template <bool FF>
struct ChunkSum;
template <>
struct ChunkSum<false> {
    double v;
    __device__ __forceinline__ void zero() { v = 0.0; }
    __device__ __forceinline__ void add(float c, int e) { v = fma((double)c, pow2d(e), v); }
    __device__ __forceinline__ double get() const { return v; }
};
template <>
struct ChunkSum<true> {
    float h, l;
    int R;
    __device__ __forceinline__ void zero()
    {
        h = l = 0.0f;
        R = kZeroExp;
    }
    __device__ __forceinline__ void add(float c, int e)
    {
        if (e > R) {  // warp-uniform: e is the slice exponent
            const float sc = pow2f_or_zero(R - e);
            h *= sc;
            l *= sc;
            R = e;
        }
        const float v = __fmul_rn(c, pow2f_or_zero(e - R));
        const float s = __fadd_rn(h, v);
        const float bb = __fsub_rn(s, h);
        const float err = __fadd_rn(__fsub_rn(h, __fsub_rn(s, bb)), __fsub_rn(v, bb));
        h = s;
        l = __fadd_rn(l, err);
    }
    __device__ __forceinline__ double get() const { return ldexp((double)h + (double)l, R); }
};
// The 8-slot kernels of the (0 0 0) family alone (up to 16 window sums per chunk
// against a cheap two-term recurrence) keep their sums on the FP32 pipe; the
// others keep FP64, where the FP64 pipe is not the limit and the running
// exponents would push their registers past 128 into spills.
template <int NWIN, bool N22>
constexpr bool chunk_sums_ff() { return NWIN >= 8 && !N22; }

// Window slices move in two stages.  fetch_slice issues asynchronous copies
// (cp.async, 8 bytes per lane and slot) of the raw (mantissa, exponent) slots
// [base, base + kSlots) into shared memory; they land while the previous chunk
// computes.  scale_slice then rescales the raw slice by 2^-E, with E the
// slice's largest exponent, into the FP32 slots the steps read, and returns E.
__device__ __forceinline__ void fetch_slice(int2* raw, const int2* __restrict__ bf, int base, int wlen, int lane)
{
#pragma unroll
    for (int q = 0; q < kStagePerLane; ++q) {
        const int j = base + lane + 32 * q;
        int2* d = raw + lane + 32 * q;
        if (j >= 0 && j < wlen) {
            const unsigned sa = (unsigned)__cvta_generic_to_shared(d);
            asm volatile("cp.async.ca.shared.global [%0], [%1], 8;\n" ::"r"(sa), "l"(bf + j) : "memory");
        } else {
            *d = make_int2(0, kZeroExp);
        }
    }
}
__device__ __forceinline__ void fetch_commit() { asm volatile("cp.async.commit_group;\n" ::: "memory"); }
__device__ __forceinline__ void fetch_wait_all() { asm volatile("cp.async.wait_group 0;\n" ::: "memory"); }

__device__ __forceinline__ int scale_slice(float* dst, const int2* raw, int lane, int stride = 1)
{
    int2 v[kStagePerLane];
    int emax = kZeroExp;
#pragma unroll
    for (int q = 0; q < kStagePerLane; ++q) {
        v[q] = raw[lane + 32 * q];
        emax = max(emax, v[q].y);
    }
    emax = __reduce_max_sync(0xffffffffu, emax);
#pragma unroll
    for (int q = 0; q < kStagePerLane; ++q)
        dst[(lane + 32 * q) * stride] = __int_as_float(v[q].x) * pow2f_or_zero(v[q].y - emax);
    return emax;
}

// The scaled slices of a 4-slot kernel are interleaved as [slot][window], so
// that a step reads the values of all its windows with one 16-byte load; other
// kernels keep [window][slot].  Measured: the interleaving makes the 4-slot
// kernels 0.2-4 % faster and the 8-slot ones (two 16-byte loads per step) up
// to 16 % slower.
template <int NWIN>
constexpr bool slots_interleaved() { return NWIN == 4; }

// Window configuration: 4 bits per window, product + 1 in bits 0-1 (so a used
// window is never 0) and parity in bits 2-3.  A non-zero SPEC fixes the
// product and parity of every window slot at compile time (the common
// mode-coupling and covariance sets); the number of used slots stays a launch
// parameter (p.nwin <= NWIN), so one instantiation serves every prefix of its
// slot list.  SPEC == 0 reads the configuration from the launch parameters.
__host__ __device__ constexpr uint32_t wspec(int prod, int par) { return (uint32_t)((prod + 1) | (par << 2)); }
template <uint32_t SPEC>
__device__ __forceinline__ int wprod(const CouplingParams& p, int k)
{
    return SPEC ? (int)((SPEC >> (4 * k)) & 3u) - 1 : p.win[k].product;
}
template <uint32_t SPEC>
__device__ __forceinline__ int wpar(const CouplingParams& p, int k)
{
    return SPEC ? (int)((SPEC >> (4 * k + 2)) & 3u) : p.win[k].parity;
}

// Per-direction recurrence state (float-float values; the 22 family is left
// unnormalised between steps, see ff_add_raw).
// n copies of one slot spec w (4 bits) in consecutive slots
__host__ __device__ constexpr uint32_t rep(uint32_t w, int n) { return n == 0 ? 0u : (w | (rep(w, n - 1) << 4)); }
constexpr uint32_t W00 = wspec(PROD_00_00, PAR_ALL), W02 = wspec(PROD_00_22, PAR_EVEN);
constexpr uint32_t WPP = wspec(PROD_22_22, PAR_EVEN), WMM = wspec(PROD_22_22, PAR_ODD);
// the window sets of the mode-coupling and covariance entry points
constexpr uint32_t S_MCM4 = W00 | (W02 << 4) | (WPP << 8) | (WMM << 12);
constexpr uint32_t S_PPMM = WPP | (WMM << 4);
constexpr uint32_t S_PPMM2 = S_PPMM | (S_PPMM << 8);  // (++, --) of two windows
constexpr uint32_t S_PPMM4 = S_PPMM2 | (S_PPMM2 << 16);  // (++, --) of four windows
constexpr uint32_t S_MCM8 = S_MCM4 | (S_MCM4 << 16);     // TT, TE, ++, -- of two windows
static_assert(((S_PPMM2 >> 8) & 0xffu) == S_PPMM && ((S_PPMM2 >> 4) & 0xfu) == WMM, "slot layout of S_PPMM2");
constexpr uint32_t S_TETE = W02 | (W00 << 4) | (W02 << 8) | (W02 << 12) | (W02 << 16);

struct Sweep {
    ff f2, f2o;   // 22 family at the current point and at the previous one
    ff f0;        // 00 family at the last even point
    float w;      // ws (2j + 1) at the current point, ws = 4 or 1 (exact in FP32)
};

// The window configuration one task uses, read from the parameters once: the
// inner loops then never reload launch parameters (which, when they live in
// shared memory, the compiler could not keep in registers across the loop's
// shared-memory stores).
template <int NWIN>
struct WinCfg {
    int nwin;
    int prod[NWIN], par[NWIN];
};

template <int NWIN, uint32_t SPEC>
__device__ __forceinline__ WinCfg<NWIN> win_cfg(const CouplingParams& p)
{
    WinCfg<NWIN> c;
    c.nwin = p.nwin;
#pragma unroll
    for (int k = 0; k < NWIN; ++k) {
        c.prod[k] = wprod<SPEC>(p, k);
        c.par[k] = wpar<SPEC>(p, k);
    }
    return c;
}

template <int NWIN, bool N00, bool N22, uint32_t SPEC, bool EVEN>
__device__ __forceinline__ void sweep_acc(const WinCfg<NWIN>& p, const Sweep& s, const float* sw, int slot,
                                          float* c, float& n0, float& n2)
{
    float wv[NWIN];  // this slot's scaled value of each window
    if constexpr (slots_interleaved<NWIN>()) {  // sw is 16-byte aligned (the callers' __align__(16) arrays)
        const float4 t = *reinterpret_cast<const float4*>(sw + slot * NWIN);
        wv[0] = t.x; wv[1] = t.y; wv[2] = t.z; wv[3] = t.w;
    } else {
#pragma unroll
        for (int k = 0; k < NWIN; ++k) wv[k] = sw[k * kSlots + slot];
    }
    const float g2 = N22 ? __fadd_rn(s.f2.h, s.f2.l) : 0.0f;  // the value rounded to one float
    float x22 = __fmul_rn(g2, g2);
    if (N22) n2 = __fmaf_rn(s.w, x22, n2);
    if (EVEN) {
        const float g0 = N00 ? __fadd_rn(s.f0.h, s.f0.l) : 0.0f;
        float x00 = __fmul_rn(g0, g0);
        float x02 = __fmul_rn(g0, g2);
        if (N00) n0 = __fmaf_rn(s.w, x00, n0);
#pragma unroll
        for (int k = 0; k < NWIN; ++k) {
            if (k < p.nwin && p.par[k] != PAR_ODD) {
                const int pr = p.prod[k];
                float x = pr == PROD_00_00 ? x00 : (pr == PROD_22_22 ? x22 : x02);
                c[k] = __fmaf_rn(x, wv[k], c[k]);
            }
        }
    } else if (N22) {
#pragma unroll
        for (int k = 0; k < NWIN; ++k) {
            if (k < p.nwin && p.prod[k] == PROD_22_22 && p.par[k] != PAR_EVEN)
                c[k] = __fmaf_rn(x22, wv[k], c[k]);
        }
    }
}

// One warp task: 32 consecutive l2 from l2_0 of row l1.  sF / sB are the
// warp's shared-memory staging areas ([NWIN][kSlots] floats each).
// ---- coefficient tables ----------------------------------------------------
// For lane i of a warp task (l1, l2_0 + i) the recurrence coefficient at
// forward step t factorises as P = G(t) F(u), u = 2i + t, with
//   G(t) = t (2 l1 + 1 - t)             (the same for every lane)
//   F(u) = (2 d0 + u)(2 l2_0 + 1 + u)   (d0 = l2_0 - l1, shared along u)
// and at backward step t as P' = G'(t) F'(v), v = 2i - t, with
//   G'(t) = (2 l1 - t)(1 + t),  F'(v) = (2 l2_0 + v)(2 l1 + 2 l2_0 + 1 + v).
// So the step factors rho = a(j)/a(j+1) and 1/a(j+1) are products of a
// lane-uniform G factor and a shared F factor.  Once per chunk the warp
// tabulates these square-root ratios in shared memory (each lane a few
// entries), and every step then costs two float-float products instead of a
// float-float P, 1/sqrt(P) and a(j).  G'(t-1)/G'(t) = G(t)/G(t+1), built from
// the same two products (each commutative), so one G table serves both sweeps.
constexpr int kFEnt = kChunk / 2 + 32;  // F entries per parity of u (or v)
struct __align__(16) ffpair {
    ff rho, r;  // loaded together (one 16-byte shared load)
};
struct CoefTab {
    ffpair g[kChunk];       // sqrt(G(t)/G(t+1)), 1/sqrt(G(t+1)); both sweeps
    ffpair fF[2][kFEnt];    // forward: sqrt(F(u)/F(u+1)), 1/sqrt(F(u+1))
    ffpair fB[2][kFEnt];    // backward: sqrt(F'(v+1)/F'(v)), 1/sqrt(F'(v))
};

// rho = sqrt(X / Y) for X >= 0, Y > 0 (float-float); 0 for X = 0
__device__ __forceinline__ ff sqrt_ratio_rho(ff X, ff Y)
{
    return X.h > 0.0f ? ff_mul(X, ff_rsqrt(ff_mul_raw(X, Y))) : ff_make(0.0f);
}
// rho as above and r = 1 / sqrt(Y)
__device__ __forceinline__ void sqrt_ratio(ff X, ff Y, ff& rho, ff& r)
{
    r = ff_rsqrt(Y);
    rho = sqrt_ratio_rho(X, Y);
}

// F entry e of the chunk at t0: forward u = t0 + e, backward v = e - t0 - 31.
__device__ __forceinline__ void f_fwd(CoefTab& tb, int e, int t0, int l1, int l2_0)
{
    const int d0 = l2_0 - l1;
    const float u = (float)(t0 + e);
    const ff X = two_prod((float)(2 * d0) + u, (float)(2 * l2_0 + 1) + u);
    const ff Y = two_prod((float)(2 * d0 + 1) + u, (float)(2 * l2_0 + 2) + u);
    ff a, b;
    sqrt_ratio(X, Y, a, b);
    tb.fF[e & 1][e >> 1] = ffpair{a, b};
}
__device__ __forceinline__ void f_bwd(CoefTab& tb, int e, int t0, int l1, int l2_0)
{
    const int v = e - t0 - (kChunk - 1);
    const float fv = (float)v;
    ff a = ff_make(0.0f), b = ff_make(0.0f);
    if (2 * l2_0 + v > 0)
        sqrt_ratio(two_prod((float)(2 * l2_0 + 1) + fv, (float)(2 * l1 + 2 * l2_0 + 2) + fv),
                   two_prod((float)(2 * l2_0) + fv, (float)(2 * l1 + 2 * l2_0 + 1) + fv), a, b);
    tb.fB[e & 1][e >> 1] = ffpair{a, b};
}
// Without the (2 -2 0) family only the odd steps of the (0 0 0) recurrence use
// the tables, and only rho: odd e forward (fF[1]) and even e backward (fB[0]).
// Lanes of odd e form a forward entry and lanes of even e a backward one, from
// operands selected per lane, with one shared sqrt_ratio_rho.
__device__ __forceinline__ void f_rho_odd_steps(CoefTab& tb, int e, int t0, int l1, int l2_0)
{
    const bool fwd = e & 1;
    const int d0 = l2_0 - l1;
    const float u = (float)(t0 + e);
    const int v = e - t0 - (kChunk - 1);
    const float fv = (float)v;
    const float x1 = fwd ? (float)(2 * d0) + u : (float)(2 * l2_0 + 1) + fv;
    const float x2 = fwd ? (float)(2 * l2_0 + 1) + u : (float)(2 * l1 + 2 * l2_0 + 2) + fv;
    const float y1 = fwd ? (float)(2 * d0 + 1) + u : (float)(2 * l2_0) + fv;
    const float y2 = fwd ? (float)(2 * l2_0 + 2) + u : (float)(2 * l1 + 2 * l2_0 + 1) + fv;
    ff rho = sqrt_ratio_rho(two_prod(x1, x2), two_prod(y1, y2));
    if (!fwd && 2 * l2_0 + v <= 0) rho = ff_make(0.0f);
    (fwd ? tb.fF[1][e >> 1] : tb.fB[0][e >> 1]).rho = rho;
}

// The F entries of a task's first chunk (t0 = 0), formed in full.
template <bool N22>
__device__ __forceinline__ void init_f_tables(CoefTab& tb, int l1, int l2_0, int lane)
{
#pragma unroll
    for (int q = 0; q < 2 * kFEnt / 32; ++q) {
        const int e = lane + 32 * q;
        if (N22) {
            f_fwd(tb, e, 0, l1, l2_0);
            f_bwd(tb, e, 0, l1, l2_0);
        } else {
            f_rho_odd_steps(tb, e, 0, l1, l2_0);
        }
    }
}

// One in-place move of a table row by 16 entries: every lane reads before any writes.
__device__ __forceinline__ void move_row(ffpair* row, int from, int to)
{
    const ffpair x = row[from];
    __syncwarp();
    row[to] = x;
}

// The tables of the chunk at t0.  The G entries are formed anew each chunk.
// The F entries of the first chunk come from init_f_tables; after that 64 of
// the 96 entries per sweep are the previous chunk's moved by 32 in e (16 per
// parity: forward down, backward up), and only 32 are new.
template <bool N22>
__device__ __forceinline__ void build_tables(CoefTab& tb, int t0, int T, int l1, int l2_0, int lane)
{
    const ff zero = ff_make(0.0f);
    {
        const int ti = t0 + lane;
        const float t = (float)ti;
        ff a = zero, b = zero;
        if (ti < T) {
            const ff X = two_prod(t, (float)(2 * l1 + 1) - t), Y = two_prod(t + 1.0f, (float)(2 * l1) - t);
            if (N22) sqrt_ratio(X, Y, a, b);
            else a = sqrt_ratio_rho(X, Y);
        }
        tb.g[lane] = ffpair{a, b};
    }
    if (t0 == 0) return;
    static_assert(2 * kFEnt == 96 && kChunk == 32, "the move below assumes 96 F entries and 32-step chunks");
    if (N22) {
        move_row(tb.fF[0], lane + 16, lane);
        move_row(tb.fF[1], lane + 16, lane);
        move_row(tb.fB[0], lane, lane + 16);
        move_row(tb.fB[1], lane, lane + 16);
        f_fwd(tb, 64 + lane, t0, l1, l2_0);
        f_bwd(tb, lane, t0, l1, l2_0);
    } else {
        move_row(tb.fF[1], lane + 16, lane);
        move_row(tb.fB[0], lane, lane + 16);
        f_rho_odd_steps(tb, (lane & 1) ? 64 + lane : lane, t0, l1, l2_0);
    }
}

// One table-driven step: f(next) = -(4 (2j+1) f(cur) r + rho f(prev)).  With
// WS4 the sweep carries w = 4 (2j+1) and the step saves the multiply by 4.
// Both forms give the same bits (4 (2j+1) is exact); which one a slot list
// uses is a measured choice: the compiler schedules the all-spins list
// (S_MCM4) about 1 % faster without it and every other list 1-3 % faster
// with it.
template <int NWIN, uint32_t SPEC>
constexpr bool weight_times4() { return !(NWIN == 4 && SPEC == S_MCM4); }
template <bool N00, bool N22, bool ODD_STEP, bool WS4>
__device__ __forceinline__ void tab_step(Sweep& s, ff rho, ff r, float dw)
{
    if (N22) {
        ff u = ff_mul_raw(ff_mulf_raw(s.f2, WS4 ? s.w : 4.0f * s.w), r);
        ff v = ff_mul_raw(rho, s.f2o);
        ff nf = ff_neg(ff_add_raw(u, v));
        s.f2o = s.f2;
        s.f2 = nf;
    }
    if (N00 && ODD_STEP) s.f0 = ff_neg(ff_mul_raw(rho, s.f0));
    s.w += dw;
}

template <bool N00, bool N22, bool ODD_STEP, bool WS4>
__device__ __forceinline__ void tab_fwd(Sweep& s, const CoefTab& tb, int st, int lane)
{
    const int e = lane + (st >> 1);  // (u - t0) / 2; u - t0 = 2 lane + st has the parity of the step
    const ffpair g = tb.g[st], f = tb.fF[ODD_STEP][e];
    ff rho = ff_mul_raw(g.rho, f.rho);
    ff r = ff_mul_raw(g.r, f.r);
    tab_step<N00, N22, ODD_STEP, WS4>(s, rho, r, WS4 ? 8.0f : 2.0f);
}

template <bool N00, bool N22, bool ODD_STEP, bool WS4>
__device__ __forceinline__ void tab_bwd(Sweep& s, const CoefTab& tb, int st, int lane)
{
    // v - (-t0 - 31) = 2 lane - st + 31: odd for even steps, half of it lane + 15 - st / 2
    const int e = lane + (kChunk / 2 - 1) - (st >> 1);
    const ffpair g = tb.g[st], f = tb.fB[!ODD_STEP][e];
    ff rho = ff_mul_raw(g.rho, f.rho);
    ff r = ff_mul_raw(g.r, f.r);
    tab_step<N00, N22, ODD_STEP, WS4>(s, rho, r, WS4 ? -8.0f : -2.0f);
}

// The Xi of pair (l1, l2_0 + lane) into Xi[]; returns whether the lane holds a
// pair to write (l1 <= l2 <= lmax).  Lanes outside clamp l2 into [l1, lmax] and
// compute values nobody writes.
template <int NWIN, bool N00, bool N22, uint32_t SPEC>
__device__ __forceinline__ bool chosen_xi(const CouplingParams& p, const int l1, const int l2_0, float* sF,
                                          float* sB, int2* raw, CoefTab& tb, const int lane, double* Xi)
{
    const int l2raw = l2_0 + lane;
    const bool active = l2raw >= l1 && l2raw <= p.lmax;
    const int l2 = l2raw > p.lmax ? p.lmax : (l2raw < l1 ? l1 : l2raw);
    const int d = l2 - l1;
    const int jmin = d, jmax = l1 + l2;
    const int T = l1;
    const bool fam22 = N22 && (l1 >= 2);
    const int jmin0 = l2_0 - l1, jmax0 = l2_0 + l1;  // lane 0's ends: lane i reads slot i + step
    const WinCfg<NWIN> wc = win_cfg<NWIN, SPEC>(p);

    if (T == 0) {
        xi_single_term(p, l2, Xi);
        return active;
    }

    Sweep F, B;
    F.f2 = ff_make(1.0f); F.f2o = ff_make(0.0f); F.f0 = ff_make(1.0f);
    constexpr bool WS4 = weight_times4<NWIN, SPEC>();
    constexpr int ws = WS4 ? 4 : 1;  // the norm sums below carry this factor
    F.w = (float)(ws * (2 * jmin + 1));
    B.f2 = ff_make(1.0f); B.f2o = ff_make(0.0f); B.f0 = ff_make(1.0f);
    B.w = (float)(ws * (2 * jmax + 1));
    constexpr bool FFS = chunk_sums_ff<NWIN, N22>();
    ChunkSum<FFS> SFW[NWIN], SBW[NWIN], SFN0, SFN2, SBN0, SBN2;
#pragma unroll
    for (int k = 0; k < NWIN; ++k) {
        SFW[k].zero();
        SBW[k].zero();
    }
    SFN0.zero();
    SFN2.zero();
    SBN0.zero();
    SBN2.zero();

    int2* rF = raw;                  // raw forward slices, [NWIN][kSlots]
    int2* rB = raw + NWIN * kSlots;  // raw backward slices
#pragma unroll
    for (int k = 0; k < NWIN; ++k) {
        if (k < p.nwin) {
            fetch_slice(rF + k * kSlots, p.win[k].bf, jmin0, p.wlen, lane);
            fetch_slice(rB + k * kSlots, p.win[k].bf, jmax0 - kChunk + 1, p.wlen, lane);
        }
    }
    fetch_commit();
    init_f_tables<N22>(tb, l1, l2_0, lane);
    for (int t0 = 0; t0 < T; t0 += kChunk) {
        int eF[NWIN], eB[NWIN];
        fetch_wait_all();
        __syncwarp();
#pragma unroll
        for (int k = 0; k < NWIN; ++k) {
            if (k < p.nwin) {
                if constexpr (slots_interleaved<NWIN>()) {
                    eF[k] = scale_slice(sF + k, rF + k * kSlots, lane, NWIN);
                    eB[k] = scale_slice(sB + k, rB + k * kSlots, lane, NWIN);
                } else {
                    eF[k] = scale_slice(sF + k * kSlots, rF + k * kSlots, lane);
                    eB[k] = scale_slice(sB + k * kSlots, rB + k * kSlots, lane);
                }
            } else {
                eF[k] = eB[k] = kZeroExp;
            }
        }
        build_tables<N22>(tb, t0, T, l1, l2_0, lane);
        __syncwarp();
        if (t0 + kChunk < T) {  // the next chunk's slices land while this one computes
#pragma unroll
            for (int k = 0; k < NWIN; ++k) {
                if (k < p.nwin) {
                    fetch_slice(rF + k * kSlots, p.win[k].bf, jmin0 + t0 + kChunk, p.wlen, lane);
                    fetch_slice(rB + k * kSlots, p.win[k].bf, jmax0 - t0 - 2 * kChunk + 1, p.wlen, lane);
                }
            }
        }
        fetch_commit();
        float cF[NWIN], cB[NWIN];
#pragma unroll
        for (int k = 0; k < NWIN; ++k) cF[k] = cB[k] = 0.0f;
        float n0F = 0.0f, n2F = 0.0f, n0B = 0.0f, n2B = 0.0f;
        const int steps = min(kChunk, T - t0);  // t0 is even, so step s has the parity of s
        int s = 0;
        for (; s + 1 < steps; s += 2) {
            sweep_acc<NWIN, N00, N22, SPEC, true>(wc, F, sF, lane + s, cF, n0F, n2F);
            sweep_acc<NWIN, N00, N22, SPEC, true>(wc, B, sB, lane - s + kChunk - 1, cB, n0B, n2B);
            tab_fwd<N00, N22, false, WS4>(F, tb, s, lane);
            tab_bwd<N00, N22, false, WS4>(B, tb, s, lane);
            sweep_acc<NWIN, N00, N22, SPEC, false>(wc, F, sF, lane + s + 1, cF, n0F, n2F);
            sweep_acc<NWIN, N00, N22, SPEC, false>(wc, B, sB, lane - s - 1 + kChunk - 1, cB, n0B, n2B);
            tab_fwd<N00, N22, true, WS4>(F, tb, s + 1, lane);
            tab_bwd<N00, N22, true, WS4>(B, tb, s + 1, lane);
        }
        if (s < steps) {  // one even step left (T odd, last chunk)
            sweep_acc<NWIN, N00, N22, SPEC, true>(wc, F, sF, lane + s, cF, n0F, n2F);
            sweep_acc<NWIN, N00, N22, SPEC, true>(wc, B, sB, lane - s + kChunk - 1, cB, n0B, n2B);
            tab_fwd<N00, N22, false, WS4>(F, tb, s, lane);
            tab_bwd<N00, N22, false, WS4>(B, tb, s, lane);
        }
        // ---- flush of the chunk sums (the norm sums carry the weight factor ws = 2^(WS4 ? 2 : 0)) ----
#pragma unroll
        for (int k = 0; k < NWIN; ++k) {
            SFW[k].add(cF[k], eF[k]);
            SBW[k].add(cB[k], eB[k]);
        }
        if (N00) {
            SFN0.add(n0F, WS4 ? -2 : 0);
            SBN0.add(n0B, WS4 ? -2 : 0);
        }
        if (N22) {
            SFN2.add(n2F, WS4 ? -2 : 0);
            SBN2.add(n2B, WS4 ? -2 : 0);
        }
        __syncwarp();
    }
    double FW[NWIN], BW[NWIN];
#pragma unroll
    for (int k = 0; k < NWIN; ++k) {
        FW[k] = SFW[k].get();
        BW[k] = SBW[k].get();
    }
    double FN0 = SFN0.get(), FN2 = SFN2.get(), BN0 = SBN0.get(), BN2 = SBN2.get();

    // last forward point t = T (j = jm), in FP64; its parity is that of T
    const int jm = jmin + T;
    const bool evenT = (T & 1) == 0;
    {
        double g2d = ff_to_double(F.f2), g0d = (N00 && evenT) ? ff_to_double(F.f0) : 0.0;
        double x22 = g2d * g2d, x00 = g0d * g0d, x02 = g0d * g2d, w = 2.0 * jm + 1.0;
        if (N22) FN2 = fma(w, x22, FN2);
        if (N00) FN0 = fma(w, x00, FN0);
#pragma unroll
        for (int k = 0; k < NWIN; ++k) {
            if (k < p.nwin) {
                const int pr = wprod<SPEC>(p, k), pa = wpar<SPEC>(p, k);
                double ww = __ldg(p.win[k].wW + jm);
                if (evenT && pa != PAR_ODD)
                    FW[k] = fma(pr == PROD_00_00 ? x00 : (pr == PROD_22_22 ? x22 : x02), ww, FW[k]);
                else if (!evenT && pr == PROD_22_22 && pa != PAR_EVEN)
                    FW[k] = fma(x22, ww, FW[k]);
            }
        }
    }
    // one more forward step for g(jm + 1) (and the 00 value at jm + 1 when T is odd)
    const double gm0 = ff_to_double(F.f2);
    double gm1 = 0.0, g0s;
    {
        // P(jm) = T(2d+T)(2l1+1-T)(2l2+1+T), P(jm+1) = (T+1)(2d+T+1)(2l1-T)(2l2+2+T)
        const float fT = (float)T;
        ff P0 = ff_mul_raw(two_prod(fT, (float)(2 * d) + fT), two_prod((float)(2 * l1 + 1) - fT, (float)(2 * l2 + 1) + fT));
        ff P1 = ff_mul_raw(two_prod(fT + 1.0f, (float)(2 * d + 1) + fT), two_prod((float)(2 * l1) - fT, (float)(2 * l2 + 2) + fT));
        ff rho, r;
        sqrt_ratio(P0, P1, rho, r);
        if (N22) gm1 = ff_to_double(ff_neg(ff_add(ff_mul_raw(ff_mul_raw(F.f2, ff_make(WS4 ? F.w : 4.0f * F.w)), r), ff_mul_raw(rho, F.f2o))));
        g0s = (N00 && !evenT) ? ff_to_double(ff_neg(ff_mul(rho, F.f0))) : ff_to_double(F.f0);
    }

    const double hm0 = ff_to_double(B.f2), hm1 = ff_to_double(B.f2o), h0s = ff_to_double(B.f0);

    // match, normalise, sign (FP64)
    const double lam0 = N00 ? g0s / h0s : 0.0;
    const double lam2 = fam22 ? (gm0 * hm0 + gm1 * hm1) / (hm0 * hm0 + hm1 * hm1) : 0.0;
    const double N0 = fma(lam0 * lam0, BN0, FN0);
    const double N2 = fma(lam2 * lam2, BN2, FN2);
    const double inv0 = N00 ? kInv4Pi / N0 : 0.0;
    const double inv2 = fam22 ? kInv4Pi / N2 : 0.0;
    double inv02 = 0.0;
    if (N00 && fam22) inv02 = (((lam0 < 0.0) != (lam2 < 0.0)) ? -kInv4Pi : kInv4Pi) * rsqrt(N0 * N2);
#pragma unroll
    for (int k = 0; k < kMaxWin; ++k) {
        Xi[k] = 0.0;
        if (k < NWIN && k < p.nwin) {
            const int pr = wprod<SPEC>(p, k);
            if (pr == PROD_00_00)
                Xi[k] = fma(lam0 * lam0, BW[k], FW[k]) * inv0;
            else if (!fam22)
                Xi[k] = 0.0;
            else if (pr == PROD_22_22)
                Xi[k] = fma(lam2 * lam2, BW[k], FW[k]) * inv2;
            else
                Xi[k] = fma(lam0 * lam2, BW[k], FW[k]) * inv02;
        }
    }
    return active;
}

// One warp task with its own writes (the persistent batch kernel, whose items
// hold l2_0 >= l1).
template <int NWIN, bool N00, bool N22, uint32_t SPEC>
__device__ __forceinline__ void chosen_task(const CouplingParams& p, const int l1, const int l2_0, float* sF,
                                            float* sB, int2* raw, CoefTab& tb, const int lane)
{
    double Xi[kMaxWin];
    if (chosen_xi<NWIN, N00, N22, SPEC>(p, l1, l2_0, sF, sB, raw, tb, lane, Xi)) write_pair(p, l1, l2_0 + lane, Xi);
}


template <int NWIN, bool N00, bool N22, uint32_t SPEC>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, NWIN <= 4 ? 5 : 4) k_coupling_chosen(const CouplingParams p)
{
    __shared__ __align__(16) float sW[kWarpsPerBlock][2][NWIN][kSlots];
    __shared__ int2 sR[kWarpsPerBlock][2][NWIN][kSlots];
    __shared__ CoefTab sT[kWarpsPerBlock];
    __shared__ TileRows rows;
    const int warp = threadIdx.x >> 5, lane = threadIdx.x & 31;
    // the task list is tiled: kTileRows tasks per block, rows outside [lmin, lmax] as l1 = -1
    const int gw = (int)(blockIdx.x * (unsigned)kWarpsPerBlock) + warp;
    const int2 task = gw < p.ntasks ? p.tasks[gw] : make_int2(-1, 0);
    double Xi[kMaxWin];
    bool active = false;
    if (task.x >= 0)  // warp-uniform
        active = chosen_xi<NWIN, N00, N22, SPEC>(p, task.x, task.y, &sW[warp][0][0][0], &sW[warp][1][0][0],
                                                 &sR[warp][0][0][0], sT[warp], lane, Xi);
    // each warp's slice staging area (2 NWIN kSlots floats) holds its [NWIN][32] row-half doubles
    static_assert(2 * NWIN * kSlots >= 2 * NWIN * 32, "row-half staging fits the slice area");
    write_tile<NWIN>(p, task.x, task.y, active, Xi, reinterpret_cast<double*>(&sW[0][0][0][0]), NWIN * kSlots, rows,
                     warp, lane);
}

// families a compile-time window set needs
constexpr bool spec_needs(uint32_t spec, int nwin, bool fam00)
{
    bool need = false;
    for (int k = 0; k < nwin; ++k) {
        int pr = (int)((spec >> (4 * k)) & 3u) - 1;
        need = need || (fam00 ? pr != PROD_22_22 : pr != PROD_00_00);
    }
    return need;
}

template <int NWIN, uint32_t SPEC>
inline cudaError_t launch_cfg(const CouplingParams& p, bool n00, bool n22, cudaStream_t s)
{
    const int threads = kWarpsPerBlock * 32;
    const unsigned blocks = (unsigned)((p.ntasks + kWarpsPerBlock - 1) / kWarpsPerBlock);
    if constexpr (SPEC != 0) {
        constexpr bool a = spec_needs(SPEC, NWIN, true), b = spec_needs(SPEC, NWIN, false);
        (void)n00;
        (void)n22;
        k_coupling_chosen<NWIN, a, b, SPEC><<<blocks, threads, 0, s>>>(p);
    } else {
        if (n00 && n22)
            k_coupling_chosen<NWIN, true, true, 0><<<blocks, threads, 0, s>>>(p);
        else if (n22)
            k_coupling_chosen<NWIN, false, true, 0><<<blocks, threads, 0, s>>>(p);
        else
            k_coupling_chosen<NWIN, true, false, 0><<<blocks, threads, 0, s>>>(p);
    }
    return cudaGetLastError();
}


// True when the first `nwin` slots of `spec` equal those of the template T.
inline bool spec_fits(uint32_t spec, int nwin, uint32_t T, int TN)
{
    if (nwin > TN) return false;
    for (int k = 0; k < nwin; ++k)
        if (((spec >> (4 * k)) & 0xfu) != ((T >> (4 * k)) & 0xfu)) return false;
    return true;
}

inline uint32_t spec_of(const CouplingParams& p)
{
    uint32_t spec = 0;
    for (int k = 0; k < p.nwin && k < 8; ++k) spec |= wspec(p.win[k].product, p.win[k].parity) << (4 * k);
    return spec;
}

}  // namespace ps
