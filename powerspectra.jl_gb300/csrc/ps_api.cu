// ps_api.cu -- the C ABI (include/powerspectra_gpu.h): context, argument
// checks, device buffers, host<->device copies and kernel dispatch.
//
// Every entry point validates its arguments on the host before any device
// work, so a bad size or pointer is reported as PS_ERR_ARG and never reaches
// a kernel.
#include <stdarg.h>
#include <stdio.h>
#include <string.h>

#include <algorithm>
#include <thread>
#include <vector>

#include "ps_internal.cuh"
#include "ps_tiles.h"

// Dense solves (ps_linalg.cu)
struct ps_linalg;
ps_linalg* ps_linalg_new();
void ps_linalg_free(ps_linalg* L);
int ps_linalg_decouple(ps_linalg* L, const double* Y, const double* B1, const double* B2, int n, int64_t ldin,
                       double* out, int64_t ldout, cudaStream_t s, char* err, size_t errn, bool on_device);
int ps_linalg_solve(ps_linalg* L, const double* M, int n, int64_t ldm, const double* b, int nrhs, int64_t ldb,
                    double* x, int64_t ldx, cudaStream_t s, char* err, size_t errn);

// Largest lmax the kernels accept: the integer products in P(j) stay below 2^63
// and every index stays in 32 bits.
#define PS_MAX_LMAX 16383

struct ps_ctx {
    int device = 0;
    cudaStream_t own_stream = nullptr;
    cudaStream_t stream = nullptr;
    char err[512] = {0};
    // warp task lists for the current (lmin, lmax): rows for the plain kernel,
    // tiles for the chosen kernel
    int2* d_tasks = nullptr;
    size_t tasks_cap = 0;
    int ntasks = 0, task_lmin = -1, task_lmax = -1;
    int2* d_tiles = nullptr;
    size_t tiles_cap = 0;
    int ntiles = 0, tile_lmin = -1, tile_lmax = -1;
    // padded windows, raw inputs, spectra, outputs (element counts)
    double* d_win = nullptr;
    size_t win_cap = 0;
    double* d_raw = nullptr;
    size_t raw_cap = 0;
    double* d_spec = nullptr;
    size_t spec_cap = 0;
    double* d_out = nullptr;
    size_t out_cap = 0;
    double* d_probe = nullptr;
    int2* d_bf = nullptr;  // split (mantissa, exponent) windows for the chosen kernel
    size_t bf_cap = 0;
    double* d_alm = nullptr;  // harmonic coefficients copied in by ps_window_W (2 doubles each)
    size_t alm_cap = 0;
    double* d_part = nullptr;  // alm2cl partial sums
    size_t part_cap = 0;
    double* d_qp = nullptr;  // chosen QuickPol scratch: W as floats and its exponent
    size_t qp_cap = 0;
    // covariance sets: the windows of the tensor-core launches (padded, split) and their Xi
    double* d_cwin = nullptr;
    size_t cwin_cap = 0;
    int2* d_cbf = nullptr;
    size_t cbf_cap = 0;
    double* d_xi = nullptr;
    size_t xi_cap = 0;
    double* h_pack = nullptr;  // pinned host staging for packed coefficient sets
    size_t pack_cap = 0;
    // batched workload state (ps_batch_*)
    struct Batch {
        bool ready = false;
        int nitems = 0, npreps = 0, max_wlen = 0, group_slots = 4, blocks = 0;
        ps::CouplingParams* d_groups = nullptr;
        int4* d_items = nullptr;
        ps::WinPrep* d_preps = nullptr;
        unsigned* d_counter = nullptr;
        double* d_win = nullptr;
        int2* d_bf = nullptr;
        cudaGraphExec_t exec = nullptr;
        // one-launch-per-group form: the groups' parameters on the host, with
        // task lists per (lmin, lmax) in d_tasks
        bool launches = false;
        std::vector<ps::CouplingParams> host_groups;
        int2* d_tasks = nullptr;
        // tensor-core launches (the problems' TT slots and ++/-- slots when there are
        // mma_min_slots of them), enqueued before the CUDA-core part,
        // with the block lists of every distinct (lmin, lmax) in d_mtiles
        std::vector<ps::MmaParams> host_mma;
        std::vector<char> host_mma00;
        int2* d_mtiles = nullptr;
        unsigned char* d_btab = nullptr;  // the tensor-core launches' table of B tiles (one at a time)
    } batch;
    int tuned_group_slots = 0, tuned_blocks_per_sm = 0;
    // tensor-core kernels: their block list for the current (lmin, lmax) and the status of their bounded waits
    int2* d_mtiles = nullptr;
    size_t mtiles_cap = 0;
    int nmtiles = 0, mtile_lmin = -1, mtile_lmax = -1;
    unsigned char* d_btab = nullptr;  // their table of B tiles (mma_table_bytes), one launch at a time
    size_t btab_cap = 0;
    unsigned* d_status = nullptr;
    bool status_pending = false;  // a tensor-core launch whose status is not yet checked
    bool tensor_cores = true;
    ps_linalg* la = nullptr;
    cudaEvent_t ev0 = nullptr, ev1 = nullptr;
    bool timed = false;
    double last_ms = 0.0;
    unsigned long long launches = 0;
};

static int set_err(ps_ctx* c, int code, const char* fmt, ...)
{
    if (c) {
        va_list ap;
        va_start(ap, fmt);
        vsnprintf(c->err, sizeof(c->err), fmt, ap);
        va_end(ap);
    }
    return code;
}

#define PS_CUDA(ctx, call)                                                                                  \
    do {                                                                                                    \
        cudaError_t e_ = (call);                                                                            \
        if (e_ != cudaSuccess)                                                                              \
            return set_err((ctx), e_ == cudaErrorMemoryAllocation ? PS_ERR_OOM : PS_ERR_CUDA, "%s: %s (%s:%d)", \
                           #call, cudaGetErrorString(e_), __FILE__, __LINE__);                               \
    } while (0)

static int ensure(ps_ctx* c, double** p, size_t* cap, size_t need)
{
    if (need <= *cap) return PS_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc((void**)p, need * sizeof(double));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return set_err(c, PS_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", need * sizeof(double),
                       cudaGetErrorString(e));
    }
    *cap = need;
    return PS_OK;
}

static int ensure_pinned(ps_ctx* c, size_t need)
{
    if (need <= c->pack_cap) return PS_OK;
    cudaFreeHost(c->h_pack);
    c->h_pack = nullptr;
    c->pack_cap = 0;
    cudaError_t e = cudaMallocHost((void**)&c->h_pack, need * sizeof(double));
    if (e != cudaSuccess) {
        c->h_pack = nullptr;
        cudaGetLastError();
        return set_err(c, PS_ERR_OOM, "cudaMallocHost of %zu bytes failed: %s", need * sizeof(double),
                       cudaGetErrorString(e));
    }
    c->pack_cap = need;
    return PS_OK;
}

// The plain kernel's warp tasks: rows by decreasing l1 (longest families
// first), 32 consecutive l2 per task from l2 = l1.
static void row_task_list(int lmin, int lmax, std::vector<int2>& t)
{
    t.clear();
    t.reserve((size_t)(lmax - lmin + 1) * ((lmax - lmin) / 32 + 1));
    for (int l1 = lmax; l1 >= lmin; --l1)
        for (int l2 = l1; l2 <= lmax; l2 += 32) t.push_back(make_int2(l1, l2));
}

// The chosen kernel's warp tasks, in tiles of kTileRows (one block): the
// closed-form list of ps_tiles.h.  The kernel writes each tile's row halves as
// runs of four doubles.
static void tile_task_list(int lmin, int lmax, std::vector<int2>& t)
{
    static_assert(ps::kTileRows == 4 && 32 % ps::kTileRows == 0, "tiles of four rows inside one 32-column block");
    t.clear();
    t.reserve((size_t)ps_tiles::task_count(lmin, lmax));
    ps_tiles::for_each_task(lmin, lmax, [&](int l1, int l2_0) { t.push_back(make_int2(l1, l2_0)); });
}

static int upload_tasks(ps_ctx* c, const std::vector<int2>& t, int2** d, size_t* cap)
{
    if (t.size() > *cap) {
        if (*d) cudaFree(*d);
        *d = nullptr;
        *cap = 0;
        cudaError_t e = cudaMalloc((void**)d, t.size() * sizeof(int2));
        if (e != cudaSuccess) {
            *d = nullptr;
            cudaGetLastError();
            return set_err(c, PS_ERR_OOM, "cudaMalloc of the task list failed: %s", cudaGetErrorString(e));
        }
        *cap = t.size();
    }
    PS_CUDA(c, cudaMemcpyAsync(*d, t.data(), t.size() * sizeof(int2), cudaMemcpyHostToDevice, c->stream));
    PS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PS_OK;
}

static int ensure_tasks(ps_ctx* c, int lmin, int lmax)
{
    if (c->task_lmin == lmin && c->task_lmax == lmax && c->d_tasks) return PS_OK;
    std::vector<int2> t;
    row_task_list(lmin, lmax, t);
    c->task_lmin = c->task_lmax = -1;
    if (int st = upload_tasks(c, t, &c->d_tasks, &c->tasks_cap)) return st;
    c->ntasks = (int)t.size();
    c->task_lmin = lmin;
    c->task_lmax = lmax;
    return PS_OK;
}

static int ensure_tiles(ps_ctx* c, int lmin, int lmax)
{
    if (c->tile_lmin == lmin && c->tile_lmax == lmax && c->d_tiles) return PS_OK;
    std::vector<int2> t;
    tile_task_list(lmin, lmax, t);
    c->tile_lmin = c->tile_lmax = -1;
    if (int st = upload_tasks(c, t, &c->d_tiles, &c->tiles_cap)) return st;
    c->ntiles = (int)t.size();
    c->tile_lmin = lmin;
    c->tile_lmax = lmax;
    return PS_OK;
}

namespace ps {
void mma_tile_list(int lmin, int lmax, std::vector<int2>& t);  // ps_mma.cu
}

static int ensure_bytes(ps_ctx* c, unsigned char** p, size_t* cap, size_t need);

// The tensor-core kernels' block list for (lmin, lmax) and the scratch of their table of B tiles.
static int ensure_mtiles(ps_ctx* c, int lmin, int lmax)
{
    if (int st = ensure_bytes(c, &c->d_btab, &c->btab_cap, ps::mma_table_bytes(lmax))) return st;
    if (c->mtile_lmin == lmin && c->mtile_lmax == lmax && c->d_mtiles) return PS_OK;
    std::vector<int2> t;
    ps::mma_tile_list(lmin, lmax, t);
    c->mtile_lmin = c->mtile_lmax = -1;
    if (int st = upload_tasks(c, t, &c->d_mtiles, &c->mtiles_cap)) return st;
    c->nmtiles = (int)t.size();
    c->mtile_lmin = lmin;
    c->mtile_lmax = lmax;
    return PS_OK;
}

// The status word of the tensor-core kernels' bounded waits, cleared on the stream unless a
// launch whose status is unchecked is pending.
static int alloc_status(ps_ctx* c)
{
    if (c->d_status) return PS_OK;
    cudaError_t e = cudaMalloc((void**)&c->d_status, sizeof(unsigned));
    if (e != cudaSuccess) {
        cudaGetLastError();
        c->d_status = nullptr;
        return set_err(c, PS_ERR_OOM, "cudaMalloc of the status word failed: %s", cudaGetErrorString(e));
    }
    return PS_OK;
}
static int arm_status(ps_ctx* c, cudaStream_t s)
{
    if (int st = alloc_status(c)) return st;
    if (!c->status_pending) PS_CUDA(c, cudaMemsetAsync(c->d_status, 0, sizeof(unsigned), s));
    c->status_pending = true;
    return PS_OK;
}

// Status of the tensor-core kernels' bounded waits since the last check (the
// stream must have been synchronised).
static int check_status(ps_ctx* c)
{
    if (!c->status_pending || !c->d_status) return PS_OK;
    unsigned h = 0;
    PS_CUDA(c, cudaMemcpy(&h, c->d_status, sizeof(h), cudaMemcpyDeviceToHost));
    c->status_pending = false;
    if (h) return set_err(c, PS_ERR_TIMEOUT, "a tensor-core kernel gave up waiting for its MMAs (status %u)", h);
    return PS_OK;
}

static int check_grid(ps_ctx* c, int lmin, int lmax, int64_t nW, int64_t ld)
{
    if (!c) return PS_ERR_ARG;
    if (lmin < 0 || lmax < lmin) return set_err(c, PS_ERR_ARG, "need 0 <= lmin <= lmax (got %d, %d)", lmin, lmax);
    if (lmax > PS_MAX_LMAX) return set_err(c, PS_ERR_ARG, "lmax %d exceeds the supported maximum %d", lmax, PS_MAX_LMAX);
    if (nW < 1) return set_err(c, PS_ERR_ARG, "window length nW must be >= 1 (got %lld)", (long long)nW);
    if (ld < (int64_t)(lmax - lmin + 1))
        return set_err(c, PS_ERR_ARG, "leading dimension %lld < lmax - lmin + 1 = %d", (long long)ld, lmax - lmin + 1);
    return PS_OK;
}

static int check_mode(ps_ctx* c, int mode)
{
    if (mode == PS_MODE_PLAIN_FP64 || mode == PS_MODE_CHOSEN) return PS_OK;
    return set_err(c, PS_ERR_ARG, "unknown mode %d", mode);
}

static void spin_window(int spin, int* product, int* parity)
{
    switch (spin) {
    case PS_SPIN_00: *product = ps::PROD_00_00; *parity = ps::PAR_ALL; break;
    case PS_SPIN_02: *product = ps::PROD_00_22; *parity = ps::PAR_EVEN; break;
    case PS_SPIN_PP: *product = ps::PROD_22_22; *parity = ps::PAR_EVEN; break;
    default: *product = ps::PROD_22_22; *parity = ps::PAR_ODD; break;
    }
}

namespace ps {
int cov_nwindows(int kind)
{
    static const int nw[7] = {8, 8, 4, 5, 4, 4, 2};
    return (kind >= 0 && kind < 7) ? nw[kind] : -1;
}
int cov_nratios(int kind)
{
    static const int nr[7] = {4, 4, 2, 2, 2, 2, 0};
    return (kind >= 0 && kind < 7) ? nr[kind] : -1;
}
// Family product and parity of window k of each covariance kind (src/covariance.jl:92-446).
void cov_window_spec(int kind, int k, int* product, int* parity)
{
    switch (kind) {
    case PS_COV_EEEE:
    case PS_COV_TEEE_PLANCK: *product = PROD_22_22; *parity = PAR_EVEN; break;
    case PS_COV_TEEE: *product = PROD_00_22; *parity = PAR_EVEN; break;
    case PS_COV_TETE:
        if (k == 1) { *product = PROD_00_00; *parity = PAR_ALL; }
        else { *product = PROD_00_22; *parity = PAR_EVEN; }
        break;
    default: *product = PROD_00_00; *parity = PAR_ALL; break;
    }
}
}  // namespace ps

// Launch the coupling kernel with event timing on the context stream.  A call
// that launches several groups passes first/last so that the two events
// bracket all of its coupling kernels (ps_last_kernel_ms).
static int run_coupling(ps_ctx* c, ps::CouplingParams& p, int mode, bool first = true, bool last = true)
{
    const bool chosen = mode == PS_MODE_CHOSEN;
    int st = chosen ? ensure_tiles(c, p.lmin, p.lmax) : ensure_tasks(c, p.lmin, p.lmax);
    if (st) return st;
    p.tasks = chosen ? c->d_tiles : c->d_tasks;
    p.ntasks = chosen ? c->ntiles : c->ntasks;
    if (first) PS_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    if (mode == PS_MODE_CHOSEN)
        PS_CUDA(c, ps::launch_chosen(p, c->stream));
    else
        PS_CUDA(c, ps::launch_plain_fp64(p, c->stream));
    c->launches++;
    if (last) {
        PS_CUDA(c, cudaEventRecord(c->ev1, c->stream));
        c->timed = true;
    }
    return PS_OK;
}

static int ensure_bytes(ps_ctx* c, unsigned char** p, size_t* cap, size_t need)
{
    if (need <= *cap) return PS_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc((void**)p, need);
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return set_err(c, PS_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", need, cudaGetErrorString(e));
    }
    *cap = need;
    return PS_OK;
}

static int ensure_int2(ps_ctx* c, int2** p, size_t* cap, size_t need)
{
    if (need <= *cap) return PS_OK;
    if (*p) cudaFree(*p);
    *p = nullptr;
    *cap = 0;
    cudaError_t e = cudaMalloc((void**)p, need * sizeof(int2));
    if (e != cudaSuccess) {
        *p = nullptr;
        cudaGetLastError();
        return set_err(c, PS_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", need * sizeof(int2), cudaGetErrorString(e));
    }
    *cap = need;
    return PS_OK;
}

// Upload (if host) and pad K windows into ctx->d_win; fills p.win[k].wW (and,
// for the chosen kernel, the split copies p.win[k].bf).
static int stage_windows(ps_ctx* c, ps::CouplingParams& p, const double* const* W, int K, int64_t nW, int lmax,
                         bool host, int mode)
{
    int wlen = 2 * lmax + 2;
    p.wlen = wlen;
    long long nuse = nW < (int64_t)(2 * lmax + 1) ? nW : (int64_t)(2 * lmax + 1);
    int st = ensure(c, &c->d_win, &c->win_cap, (size_t)K * wlen);
    if (st) return st;
    if (host) {
        st = ensure(c, &c->d_raw, &c->raw_cap, (size_t)K * nuse);
        if (st) return st;
    }
    for (int k = 0; k < K; ++k) {
        if (!W[k]) return set_err(c, PS_ERR_ARG, "window %d is NULL", k);
        const double* src = W[k];
        if (host) {
            PS_CUDA(c, cudaMemcpyAsync(c->d_raw + (size_t)k * nuse, W[k], nuse * sizeof(double),
                                       cudaMemcpyHostToDevice, c->stream));
            src = c->d_raw + (size_t)k * nuse;
        }
        PS_CUDA(c, ps::launch_pad_windows(c->d_win + (size_t)k * wlen, src, nuse, wlen, c->stream));
        c->launches++;
        p.win[k].wW = c->d_win + (size_t)k * wlen;
    }
    if (mode == PS_MODE_CHOSEN) {
        if ((st = ensure_int2(c, &c->d_bf, &c->bf_cap, (size_t)K * wlen))) return st;
        for (int k = 0; k < K; ++k) {
            PS_CUDA(c, ps::launch_split_windows(c->d_bf + (size_t)k * wlen, p.win[k].wW, wlen, c->stream));
            c->launches++;
            p.win[k].bf = c->d_bf + (size_t)k * wlen;
        }
    }
    return PS_OK;
}

static void batch_release(ps_ctx* c)
{
    ps_ctx::Batch& b = c->batch;
    if (b.exec) cudaGraphExecDestroy(b.exec);
    cudaFree(b.d_groups);
    cudaFree(b.d_items);
    cudaFree(b.d_preps);
    cudaFree(b.d_counter);
    cudaFree(b.d_win);
    cudaFree(b.d_bf);
    cudaFree(b.d_tasks);
    cudaFree(b.d_mtiles);
    cudaFree(b.d_btab);
    b = ps_ctx::Batch();
}

template <typename T>
static int dev_upload(ps_ctx* c, T** dst, const std::vector<T>& v)
{
    if (v.empty()) return PS_OK;
    cudaError_t e = cudaMalloc((void**)dst, v.size() * sizeof(T));
    if (e != cudaSuccess) {
        cudaGetLastError();
        *dst = nullptr;
        return set_err(c, PS_ERR_OOM, "cudaMalloc of %zu bytes failed: %s", v.size() * sizeof(T), cudaGetErrorString(e));
    }
    PS_CUDA(c, cudaMemcpyAsync(*dst, v.data(), v.size() * sizeof(T), cudaMemcpyHostToDevice, c->stream));
    return PS_OK;
}

// Split (window, case) slots of one grid into groups of at most `gs` slots.
// `used(k, s)` says whether slot (k, s) has an output.  When every selected
// slot does, the groups take the slots window by window, so the cases of one
// window (TT, TE, ++, -- of one spectrum) share a group.  A sparse set (some
// outputs NULL) is grouped by the families its slots need instead: the TT
// slots (00 family only), then the ++ and -- slots interleaved (22 family
// only; the (++, --) slot pattern has compile-time kernels whatever the
// windows), then the TE slots (both families), so no group generates a family
// that only some of its slots use.
struct Slot {
    int k, s;
};
// Fewest slots of one kind for which a chosen-mode set takes a tensor-core kernel, by lmax.
// The tensor-core kernels cost about the same for 1 to 15 windows; the CUDA-core groups grow
// with the slots, and win for small grids, where the tensor-core kernel's ramps and block
// boundaries weigh more.  Measured (ms, tensor-core against CUDA-core):
//   ++/--  lmax  511:  8 slots 0.24 / 0.17, 12 slots 0.26 / 0.31
//          lmax 1023:  8 slots 1.18 / 1.12, 12 slots 1.22 / 1.84
//          lmax 2047:  4 slots 7.4 / 5.4,   6 slots 7.4 / 7.7
//          lmax 4095:  4 slots 53 / 42,     6 slots 53 / 59
//   TT     lmax  511:  8 slots 0.138 / 0.127
//          lmax 1023:  4 slots 0.47 / 0.38, 6 slots 0.49 / 0.67
//          lmax 2047:  4 slots 2.69 / 2.54, 6 slots 2.75 / 4.21
//          lmax 4095:  3 slots 18.1 / 18.0, 4 slots 18.2 / 19.4
// On the lmax 8191 set 13 ++/-- slots take 405 ms on the tensor cores against 944 ms in two
// CUDA-core groups, and 7 TT slots 132 ms against 257 ms.
static int mma_min_slots(bool fam00, int lmax)
{
    if (fam00) return lmax >= 3072 ? 4 : (lmax >= 768 ? 5 : ps::kMaxWin + 1);
    return lmax >= 1536 ? 5 : ps::kMaxWin + 1;
}
template <typename Used>
static std::vector<std::vector<Slot>> group_slots(unsigned cases, int K, int gs, Used used)
{
    std::vector<Slot> all;
    bool dense = true;
    for (int k = 0; k < K; ++k)
        for (int s = 0; s < 4; ++s)
            if (cases & (1u << s)) {
                if (used(k, s)) all.push_back(Slot{k, s});
                else dense = false;
            }
    std::vector<std::vector<Slot>> out;
    auto chunk = [&](const std::vector<Slot>& v) {
        for (size_t i = 0; i < v.size(); i += (size_t)gs)
            out.emplace_back(v.begin() + i, v.begin() + std::min(v.size(), i + (size_t)gs));
    };
    if (dense) {
        chunk(all);
        return out;
    }
    std::vector<Slot> tt, te, pp, mm, pm;
    for (const Slot& q : all) (q.s == PS_SPIN_00 ? tt : q.s == PS_SPIN_02 ? te : q.s == PS_SPIN_PP ? pp : mm).push_back(q);
    for (size_t i = 0; i < std::max(pp.size(), mm.size()); ++i) {
        if (i < pp.size()) pm.push_back(pp[i]);
        if (i < mm.size()) pm.push_back(mm[i]);
    }
    chunk(tt);
    chunk(pm);
    chunk(te);
    return out;
}

// Batch groups hold whole windows in one of the per-window slot patterns the
// persistent kernel has a compile-time body for (TT, TE, ++, --, ++/-- pairs,
// TT/TE/++/--); any other combination of cases is split case by case.
static std::vector<std::vector<Slot>> batch_group_slots(unsigned cases, int K, int gs)
{
    std::vector<std::vector<Slot>> out;
    auto pack = [&](unsigned cs) {
        int per = __builtin_popcount(cs);
        int wpg = per >= gs ? 1 : gs / per;  // windows per group
        for (int k0 = 0; k0 < K; k0 += wpg) {
            std::vector<Slot> g;
            for (int k = k0; k < std::min(K, k0 + wpg); ++k)
                for (int s = 0; s < 4; ++s)
                    if (cs & (1u << s)) g.push_back(Slot{k, s});
            out.push_back(g);
        }
    };
    if (cases == 0x1 || cases == 0x2 || cases == 0x4 || cases == 0x8 || cases == 0xC || (cases == 0xF && gs >= 4))
        pack(cases);
    else
        for (int s = 0; s < 4; ++s)
            if (cases & (1u << s)) pack(1u << s);
    return out;
}

static int check_problem(ps_ctx* c, const ps_problem& p, int i)
{
    if (p.lmin < 0 || p.lmax < p.lmin || p.lmax > PS_MAX_LMAX)
        return set_err(c, PS_ERR_ARG, "problem %d: need 0 <= lmin <= lmax <= %d", i, PS_MAX_LMAX);
    if (p.cases == 0 || (p.cases & ~0xFu)) return set_err(c, PS_ERR_ARG, "problem %d: cases mask 0x%x", i, p.cases);
    if (p.K < 1 || !p.W || !p.M) return set_err(c, PS_ERR_ARG, "problem %d: K >= 1 and W, M arrays required", i);
    if (p.nW < 1) return set_err(c, PS_ERR_ARG, "problem %d: nW must be >= 1", i);
    if (p.ldm < p.lmax - p.lmin + 1) return set_err(c, PS_ERR_ARG, "problem %d: ldm too small", i);
    for (int k = 0; k < p.K; ++k) {
        if (!p.W[k]) return set_err(c, PS_ERR_ARG, "problem %d: W[%d] is NULL", i, k);
        for (int s = 0; s < 4; ++s)
            if ((p.cases & (1u << s)) && !p.M[4 * k + s])
                return set_err(c, PS_ERR_ARG, "problem %d: M[%d] is NULL", i, 4 * k + s);
    }
    return PS_OK;
}

extern "C" {

int ps_create(int device, ps_ctx** out)
{
    if (!out) return PS_ERR_ARG;
    *out = nullptr;
    int n = 0;
    if (cudaGetDeviceCount(&n) != cudaSuccess || n == 0) {
        cudaGetLastError();
        return PS_ERR_CUDA;
    }
    if (device < 0 || device >= n) return PS_ERR_ARG;
    ps_ctx* c = new ps_ctx();
    c->device = device;
    if (cudaSetDevice(device) != cudaSuccess || cudaStreamCreateWithFlags(&c->own_stream, cudaStreamNonBlocking) != cudaSuccess ||
        cudaEventCreate(&c->ev0) != cudaSuccess || cudaEventCreate(&c->ev1) != cudaSuccess) {
        cudaGetLastError();
        delete c;
        return PS_ERR_CUDA;
    }
    c->stream = c->own_stream;
    *out = c;
    return PS_OK;
}

void ps_destroy(ps_ctx* c)
{
    if (!c) return;
    cudaSetDevice(c->device);
    cudaStreamSynchronize(c->stream);
    cudaFree(c->d_tasks);
    cudaFree(c->d_tiles);
    cudaFree(c->d_win);
    cudaFree(c->d_raw);
    cudaFree(c->d_spec);
    cudaFree(c->d_cwin);
    cudaFree(c->d_cbf);
    cudaFree(c->d_xi);
    cudaFree(c->d_out);
    cudaFree(c->d_probe);
    cudaFree(c->d_bf);
    cudaFree(c->d_alm);
    cudaFree(c->d_part);
    cudaFree(c->d_qp);
    cudaFree(c->d_mtiles);
    cudaFree(c->d_btab);
    cudaFree(c->d_status);
    cudaFreeHost(c->h_pack);
    batch_release(c);
    ps_linalg_free(c->la);
    if (c->ev0) cudaEventDestroy(c->ev0);
    if (c->ev1) cudaEventDestroy(c->ev1);
    if (c->own_stream) cudaStreamDestroy(c->own_stream);
    delete c;
}

const char* ps_last_error(const ps_ctx* c) { return c ? c->err : "null context"; }

int ps_set_stream(ps_ctx* c, void* s)
{
    if (!c) return PS_ERR_ARG;
    c->stream = s ? (cudaStream_t)s : c->own_stream;
    return PS_OK;
}

int ps_synchronize(ps_ctx* c)
{
    if (!c) return PS_ERR_ARG;
    PS_CUDA(c, cudaSetDevice(c->device));
    PS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_status(c);
}

int ps_set_tensor_cores(ps_ctx* c, int enable)
{
    if (!c) return PS_ERR_ARG;
    c->tensor_cores = enable != 0;
    return PS_OK;
}

double ps_last_kernel_ms(const ps_ctx* c)
{
    if (!c || !c->timed) return -1.0;
    float ms = 0.f;
    if (cudaEventSynchronize(c->ev1) != cudaSuccess || cudaEventElapsedTime(&ms, c->ev0, c->ev1) != cudaSuccess) {
        cudaGetLastError();
        return -1.0;
    }
    return (double)ms;
}

uint64_t ps_launch_count(const ps_ctx* c) { return c ? (uint64_t)c->launches : 0; }

// The device address of a page-locked host buffer that is mapped into the
// device's address space (cudaHostAlloc / cudaHostRegister memory under unified
// addressing), or nullptr for ordinary pageable memory.
// Whether p (a host or device address) lies in host memory.
static bool host_resident(const void* p)
{
    cudaPointerAttributes a;
    if (!p || cudaPointerGetAttributes(&a, p) != cudaSuccess) {
        cudaGetLastError();
        return false;
    }
    return a.type == cudaMemoryTypeHost;
}

static double* mapped_host(double* h)
{
    cudaPointerAttributes a;
    if (cudaPointerGetAttributes(&a, h) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    return (a.type == cudaMemoryTypeHost && a.devicePointer) ? (double*)a.devicePointer : nullptr;
}

static int mcm_multi_impl(ps_ctx* c, unsigned cases, const double* const W[4], int64_t nW, int lmin, int lmax, int mode,
                          double* const M[4], int64_t ldm, bool host)
{
    int st = check_grid(c, lmin, lmax, nW, ldm);
    if (st) return st;
    if ((st = check_mode(c, mode))) return st;
    if (cases == 0 || (cases & ~0xFu)) return set_err(c, PS_ERR_ARG, "cases mask 0x%x must select bits 0..3", cases);
    if (!W || !M) return set_err(c, PS_ERR_ARG, "W and M arrays must not be NULL");
    PS_CUDA(c, cudaSetDevice(c->device));
    ps::CouplingParams p;
    memset(&p, 0, sizeof(p));
    p.lmin = lmin;
    p.lmax = lmax;
    p.epilogue = ps::EPI_MCM;
    const double* wsel[4];
    int sel[4], K = 0;
    for (int s = 0; s < 4; ++s) {
        if (!(cases & (1u << s))) continue;
        if (!W[s] || !M[s]) return set_err(c, PS_ERR_ARG, "spin case %d selected but its W or M pointer is NULL", s);
        spin_window(s, &p.win[K].product, &p.win[K].parity);
        wsel[K] = W[s];
        sel[K] = s;
        ++K;
    }
    p.nwin = K;
    if ((st = stage_windows(c, p, wsel, K, nW, lmax, host, mode))) return st;
    const long long n = lmax - lmin + 1;
    // Host outputs in mapped page-locked memory are written by the kernel
    // itself, so the transfer to the host overlaps the computation; pageable
    // outputs go through a device staging matrix and one copy each.
    bool direct = host;
    double* mapped[4] = {nullptr, nullptr, nullptr, nullptr};
    for (int k = 0; k < K && direct; ++k) direct = (mapped[k] = mapped_host(M[sel[k]])) != nullptr;
    if (direct) {
        for (int k = 0; k < K; ++k) p.out[k] = mapped[k];
        p.ldo = ldm;
    } else if (host) {
        if ((st = ensure(c, &c->d_out, &c->out_cap, (size_t)K * n * n))) return st;
        for (int k = 0; k < K; ++k) p.out[k] = c->d_out + (size_t)k * n * n;
        p.ldo = n;
    } else {
        for (int k = 0; k < K; ++k) p.out[k] = M[sel[k]];
        p.ldo = ldm;
    }
    if ((st = run_coupling(c, p, mode))) return st;
    if (direct) {
        PS_CUDA(c, cudaStreamSynchronize(c->stream));
    } else if (host) {
        for (int k = 0; k < K; ++k)
            PS_CUDA(c, cudaMemcpy2DAsync(M[sel[k]], (size_t)ldm * sizeof(double), p.out[k], (size_t)n * sizeof(double),
                                         (size_t)n * sizeof(double), (size_t)n, cudaMemcpyDeviceToHost, c->stream));
        PS_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return PS_OK;
}

int ps_mcm(ps_ctx* c, int spin, const double* W, int64_t nW, int lmin, int lmax, int mode, double* M, int64_t ldm)
{
    if (!c) return PS_ERR_ARG;
    if (spin < 0 || spin > 3) return set_err(c, PS_ERR_ARG, "%d is not a valid spin case", spin);
    const double* Ws[4] = {nullptr, nullptr, nullptr, nullptr};
    double* Ms[4] = {nullptr, nullptr, nullptr, nullptr};
    Ws[spin] = W;
    Ms[spin] = M;
    return mcm_multi_impl(c, 1u << spin, Ws, nW, lmin, lmax, mode, Ms, ldm, true);
}

int ps_mcm_multi(ps_ctx* c, unsigned cases, const double* const W[4], int64_t nW, int lmin, int lmax, int mode,
                 double* const M[4], int64_t ldm)
{
    return mcm_multi_impl(c, cases, W, nW, lmin, lmax, mode, M, ldm, true);
}

int ps_mcm_multi_device(ps_ctx* c, unsigned cases, const double* const dW[4], int64_t nW, int lmin, int lmax, int mode,
                        double* const dM[4], int64_t ldm)
{
    return mcm_multi_impl(c, cases, dW, nW, lmin, lmax, mode, dM, ldm, false);
}

int ps_xi(ps_ctx* c, int product, int parity, const double* const* W, int K, int64_t nW, int lmin, int lmax, int mode,
          double* const* Xi, int64_t ldx)
{
    int st = check_grid(c, lmin, lmax, nW, ldx);
    if (st) return st;
    if ((st = check_mode(c, mode))) return st;
    if (product < 0 || product > 2 || parity < 0 || parity > 2)
        return set_err(c, PS_ERR_ARG, "invalid product %d / parity %d", product, parity);
    if (K < 1 || K > ps::kMaxWin) return set_err(c, PS_ERR_ARG, "K must be in 1..%d (got %d)", ps::kMaxWin, K);
    if (!W || !Xi) return set_err(c, PS_ERR_ARG, "W and Xi arrays must not be NULL");
    for (int k = 0; k < K; ++k)
        if (!Xi[k]) return set_err(c, PS_ERR_ARG, "Xi[%d] is NULL", k);
    PS_CUDA(c, cudaSetDevice(c->device));
    ps::CouplingParams p;
    memset(&p, 0, sizeof(p));
    p.lmin = lmin;
    p.lmax = lmax;
    p.epilogue = ps::EPI_XI;
    p.nwin = K;
    for (int k = 0; k < K; ++k) {
        p.win[k].product = product;
        p.win[k].parity = parity;
    }
    if ((st = stage_windows(c, p, W, K, nW, lmax, true, mode))) return st;
    const long long n = lmax - lmin + 1;
    // page-locked outputs are written in place (then with leading dimension ldx), others staged
    bool direct = true;
    double* mapped[ps::kMaxWin] = {};
    for (int k = 0; k < K && direct; ++k) direct = (mapped[k] = mapped_host(Xi[k])) != nullptr;
    if (direct) {
        for (int k = 0; k < K; ++k) p.out[k] = mapped[k];
        p.ldo = ldx;
    } else {
        if ((st = ensure(c, &c->d_out, &c->out_cap, (size_t)K * n * n))) return st;
        for (int k = 0; k < K; ++k) p.out[k] = c->d_out + (size_t)k * n * n;
        p.ldo = n;
    }
    if ((st = run_coupling(c, p, mode))) return st;
    if (!direct)
        for (int k = 0; k < K; ++k)
            PS_CUDA(c, cudaMemcpy2DAsync(Xi[k], (size_t)ldx * sizeof(double), p.out[k], (size_t)n * sizeof(double),
                                         (size_t)n * sizeof(double), (size_t)n, cudaMemcpyDeviceToHost, c->stream));
    PS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PS_OK;
}

static int cov_impl(ps_ctx* c, int kind, const double* const* S, const double* const* R, const double* const* W,
                    int64_t nW, int lmin, int lmax, int mode, double* C, int64_t ldc, bool host, bool first = true,
                    bool last = true)
{
    int st = check_grid(c, lmin, lmax, nW, ldc);
    if (st) return st;
    if ((st = check_mode(c, mode))) return st;
    int K = ps::cov_nwindows(kind), NR = ps::cov_nratios(kind);
    if (K < 0) return set_err(c, PS_ERR_ARG, "%d is not a covariance kind", kind);
    if (!S || !W || !C || (NR > 0 && !R)) return set_err(c, PS_ERR_ARG, "S, R, W and C must not be NULL");
    for (int i = 0; i < 4; ++i)
        if (!S[i]) return set_err(c, PS_ERR_ARG, "spectrum S[%d] is NULL", i);
    for (int i = 0; i < NR; ++i)
        if (!R[i]) return set_err(c, PS_ERR_ARG, "noise ratio R[%d] is NULL", i);
    PS_CUDA(c, cudaSetDevice(c->device));
    ps::CouplingParams p;
    memset(&p, 0, sizeof(p));
    p.lmin = lmin;
    p.lmax = lmax;
    p.epilogue = ps::EPI_COV;
    p.cov_kind = kind;
    p.nwin = K;
    for (int k = 0; k < K; ++k) ps::cov_window_spec(kind, k, &p.win[k].product, &p.win[k].parity);
    if ((st = stage_windows(c, p, W, K, nW, lmax, host, mode))) return st;
    const size_t ns = (size_t)lmax + 1;
    if (host) {
        if ((st = ensure(c, &c->d_spec, &c->spec_cap, 8 * ns))) return st;
        for (int i = 0; i < 4; ++i) {
            PS_CUDA(c, cudaMemcpyAsync(c->d_spec + i * ns, S[i], ns * sizeof(double), cudaMemcpyHostToDevice, c->stream));
            p.S[i] = c->d_spec + i * ns;
        }
        for (int i = 0; i < NR; ++i) {
            PS_CUDA(c, cudaMemcpyAsync(c->d_spec + (4 + i) * ns, R[i], ns * sizeof(double), cudaMemcpyHostToDevice,
                                       c->stream));
            p.R[i] = c->d_spec + (4 + i) * ns;
        }
    } else {
        for (int i = 0; i < 4; ++i) p.S[i] = S[i];
        for (int i = 0; i < NR; ++i) p.R[i] = R[i];
    }
    const long long n = lmax - lmin + 1;
    double* mapped = host ? mapped_host(C) : nullptr;  // page-locked C: written by the kernel itself
    if (mapped) {
        p.out[0] = mapped;
        p.ldo = ldc;
    } else if (host) {
        if ((st = ensure(c, &c->d_out, &c->out_cap, (size_t)n * n))) return st;
        p.out[0] = c->d_out;
        p.ldo = n;
    } else {
        p.out[0] = C;
        p.ldo = ldc;
    }
    if ((st = run_coupling(c, p, mode, first, last))) return st;
    if (host) {
        if (!mapped)
            PS_CUDA(c, cudaMemcpy2DAsync(C, (size_t)ldc * sizeof(double), p.out[0], (size_t)n * sizeof(double),
                                         (size_t)n * sizeof(double), (size_t)n, cudaMemcpyDeviceToHost, c->stream));
        PS_CUDA(c, cudaStreamSynchronize(c->stream));
    }
    return PS_OK;
}

int ps_coupledcov(ps_ctx* c, int kind, const double* const* S, const double* const* R, const double* const* W,
                  int64_t nW, int lmin, int lmax, int mode, double* C, int64_t ldc)
{
    return cov_impl(c, kind, S, R, W, nW, lmin, lmax, mode, C, ldc, true);
}

int ps_coupledcov_device(ps_ctx* c, int kind, const double* const* dS, const double* const* dR,
                         const double* const* dW, int64_t nW, int lmin, int lmax, int mode, double* dC, int64_t ldc)
{
    return cov_impl(c, kind, dS, dR, dW, nW, lmin, lmax, mode, dC, ldc, false);
}

int ps_coupledcov_set_device(ps_ctx* c, int nblk, const int* kinds, const double* const* const* dS,
                             const double* const* const* dR, const double* const* const* dW, int64_t nW, int lmin,
                             int lmax, int mode, double* const* dC, int64_t ldc)
{
    int st = check_grid(c, lmin, lmax, nW, ldc);
    if (st) return st;
    if ((st = check_mode(c, mode))) return st;
    if (nblk < 1 || !kinds || !dS || !dW || !dC)
        return set_err(c, PS_ERR_ARG, "nblk >= 1 and the kinds, S, W and C arrays are required");
    for (int b = 0; b < nblk; ++b) {
        const int K = ps::cov_nwindows(kinds[b]), NR = ps::cov_nratios(kinds[b]);
        if (K < 0) return set_err(c, PS_ERR_ARG, "block %d: %d is not a covariance kind", b, kinds[b]);
        if (!dS[b] || !dW[b] || !dC[b] || (NR > 0 && (!dR || !dR[b])))
            return set_err(c, PS_ERR_ARG, "block %d: S, R, W and C must not be NULL", b);
        for (int i = 0; i < 4; ++i)
            if (!dS[b][i]) return set_err(c, PS_ERR_ARG, "block %d: spectrum S[%d] is NULL", b, i);
        for (int i = 0; i < NR; ++i)
            if (!dR[b][i]) return set_err(c, PS_ERR_ARG, "block %d: noise ratio R[%d] is NULL", b, i);
        for (int k = 0; k < K; ++k)
            if (!dW[b][k]) return set_err(c, PS_ERR_ARG, "block %d: window %d is NULL", b, k);
    }
    PS_CUDA(c, cudaSetDevice(c->device));
    PS_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    if (mode != PS_MODE_CHOSEN || !c->tensor_cores) {  // the fused kernel, block by block
        for (int b = 0; b < nblk; ++b)
            if ((st = cov_impl(c, kinds[b], dS[b], ps::cov_nratios(kinds[b]) > 0 ? dR[b] : nullptr, dW[b], nW, lmin,
                               lmax, mode, dC[b], ldc, false, false, false)))
                return st;
        PS_CUDA(c, cudaEventRecord(c->ev1, c->stream));
        c->timed = true;
        return PS_OK;
    }
    // Chosen mode with the tensor cores: the Xi of every window of every block, grouped across
    // the blocks by family product and parity, so that one family generation serves each group:
    // the squared (0 0 0) windows by the (0 0 0) tensor-core kernel and the squared (2 -2 0) ones
    // by the (2 -2 0) tensor-core kernel when there are mma_min_slots of them or more, and the
    // others by the CUDA-core kernel in groups of up to kMaxWin.  Then each block
    // is formed from its windows' Xi.
    struct XWin {
        int b, k, prod, par;
    };
    std::vector<XWin> xw;
    for (int b = 0; b < nblk; ++b)
        for (int k = 0; k < ps::cov_nwindows(kinds[b]); ++k) {
            XWin x{b, k, 0, 0};
            ps::cov_window_spec(kinds[b], k, &x.prod, &x.par);
            xw.push_back(x);
        }
    const int nx = (int)xw.size();
    const long long n = lmax - lmin + 1;
    const int wlen = 2 * lmax + 2;
    const long long nuse = nW < (int64_t)(2 * lmax + 1) ? nW : (int64_t)(2 * lmax + 1);
    if ((st = ensure(c, &c->d_cwin, &c->cwin_cap, (size_t)nx * wlen)) ||
        (st = ensure_int2(c, &c->d_cbf, &c->cbf_cap, (size_t)nx * wlen)) ||
        (st = ensure(c, &c->d_xi, &c->xi_cap, (size_t)nx * n * n)))
        return st;
    for (int j = 0; j < nx; ++j) {
        PS_CUDA(c, ps::launch_pad_windows(c->d_cwin + (size_t)j * wlen, dW[xw[j].b][xw[j].k], nuse, wlen, c->stream));
        PS_CUDA(c, ps::launch_split_windows(c->d_cbf + (size_t)j * wlen, c->d_cwin + (size_t)j * wlen, wlen, c->stream));
        c->launches += 2;
    }
    const int classes[4][2] = {{ps::PROD_00_00, ps::PAR_ALL}, {ps::PROD_22_22, ps::PAR_EVEN},
                               {ps::PROD_22_22, ps::PAR_ODD}, {ps::PROD_00_22, ps::PAR_EVEN}};
    for (const auto& cl : classes) {
        std::vector<int> js;
        for (int j = 0; j < nx; ++j)
            if (xw[j].prod == cl[0] && xw[j].par == cl[1]) js.push_back(j);
        if (js.empty()) continue;
        const bool mma00 = cl[0] == ps::PROD_00_00 && (int)js.size() >= mma_min_slots(true, lmax);
        const bool mma22 = cl[0] == ps::PROD_22_22 && (int)js.size() >= mma_min_slots(false, lmax);
        if (mma00 || mma22) {
            if ((st = ensure_mtiles(c, lmin, lmax)) || (st = arm_status(c, c->stream))) return st;
            for (size_t i0 = 0; i0 < js.size(); i0 += ps::kMmaMaxSlots) {
                ps::MmaParams mp;
                memset(&mp, 0, sizeof(mp));
                mp.lmin = lmin;
                mp.lmax = lmax;
                mp.nslot = (int)std::min(js.size() - i0, (size_t)ps::kMmaMaxSlots);
                for (int q = 0; q < mp.nslot; ++q) {
                    const int j = js[i0 + q];
                    mp.bf[q] = c->d_cbf + (size_t)j * wlen;
                    mp.wW[q] = c->d_cwin + (size_t)j * wlen;
                    mp.parity[q] = cl[1];
                    mp.out[q] = c->d_xi + (size_t)j * n * n;
                }
                mp.ldo = n;
                mp.wlen = wlen;
                mp.epilogue = ps::EPI_XI;
                mp.tiles = c->d_mtiles;
                mp.ntiles = c->nmtiles;
                mp.status = c->d_status;
                mp.tab = c->d_btab;
                PS_CUDA(c, ps::launch_mma(mp, mma00, c->stream));
                c->launches += 2;
            }
        } else {
            for (size_t i0 = 0; i0 < js.size(); i0 += ps::kMaxWin) {
                ps::CouplingParams p;
                memset(&p, 0, sizeof(p));
                p.lmin = lmin;
                p.lmax = lmax;
                p.epilogue = ps::EPI_XI;
                p.wlen = wlen;
                p.nwin = (int)std::min(js.size() - i0, (size_t)ps::kMaxWin);
                for (int q = 0; q < p.nwin; ++q) {
                    const int j = js[i0 + q];
                    p.win[q].product = cl[0];
                    p.win[q].parity = cl[1];
                    p.win[q].wW = c->d_cwin + (size_t)j * wlen;
                    p.win[q].bf = c->d_cbf + (size_t)j * wlen;
                    p.out[q] = c->d_xi + (size_t)j * n * n;
                }
                p.ldo = n;
                if ((st = run_coupling(c, p, mode, false, false))) return st;
            }
        }
    }
    for (int b = 0, j = 0; b < nblk; ++b) {
        ps::CovCombineParams cp;
        memset(&cp, 0, sizeof(cp));
        cp.kind = kinds[b];
        cp.lmin = lmin;
        cp.n = (int)n;
        cp.nx = ps::cov_nwindows(kinds[b]);
        for (int i = 0; i < 4; ++i) cp.S[i] = dS[b][i];
        for (int i = 0; i < ps::cov_nratios(kinds[b]); ++i) cp.R[i] = dR[b][i];
        for (int k = 0; k < cp.nx; ++k) cp.X[k] = c->d_xi + (size_t)(j + k) * n * n;
        j += cp.nx;
        cp.ldx = n;
        cp.C = dC[b];
        cp.ldc = ldc;
        PS_CUDA(c, ps::launch_cov_combine(cp, c->stream));
        c->launches++;
    }
    PS_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    c->timed = true;
    return PS_OK;
}

int ps_mcm_set_device(ps_ctx* c, unsigned cases, const double* const* dW, int K, int64_t nW, int lmin, int lmax,
                      int mode, double* const* dM, int64_t ldm)
{
    int st = check_grid(c, lmin, lmax, nW, ldm);
    if (st) return st;
    if ((st = check_mode(c, mode))) return st;
    if (cases == 0 || (cases & ~0xFu)) return set_err(c, PS_ERR_ARG, "cases mask 0x%x must select bits 0..3", cases);
    if (K < 1 || !dW || !dM) return set_err(c, PS_ERR_ARG, "K >= 1 and W, M arrays required");
    int nused = 0;
    for (int k = 0; k < K; ++k) {
        if (!dW[k]) return set_err(c, PS_ERR_ARG, "W[%d] is NULL", k);
        for (int s = 0; s < 4; ++s) nused += (cases & (1u << s)) && dM[4 * k + s];
    }
    if (nused == 0) return set_err(c, PS_ERR_ARG, "every selected output M[4k+s] is NULL");
    PS_CUDA(c, cudaSetDevice(c->device));
    // all K windows are padded (and split) once; each group points into them
    ps::CouplingParams base;
    memset(&base, 0, sizeof(base));
    base.lmin = lmin;
    base.lmax = lmax;
    base.epilogue = ps::EPI_MCM;
    base.nwin = K;
    {
        // stage_windows fills base.win[k] for k < K; it needs room for K descriptors
        std::vector<ps::WinDesc> descs(K);
        int wlen = 2 * lmax + 2;
        long long nuse = nW < (int64_t)(2 * lmax + 1) ? nW : (int64_t)(2 * lmax + 1);
        if ((st = ensure(c, &c->d_win, &c->win_cap, (size_t)K * wlen))) return st;
        if (mode == PS_MODE_CHOSEN && (st = ensure_int2(c, &c->d_bf, &c->bf_cap, (size_t)K * wlen))) return st;
        for (int k = 0; k < K; ++k) {
            PS_CUDA(c, ps::launch_pad_windows(c->d_win + (size_t)k * wlen, dW[k], nuse, wlen, c->stream));
            c->launches++;
            descs[k].wW = c->d_win + (size_t)k * wlen;
            if (mode == PS_MODE_CHOSEN) {
                PS_CUDA(c, ps::launch_split_windows(c->d_bf + (size_t)k * wlen, descs[k].wW, wlen, c->stream));
                c->launches++;
                descs[k].bf = c->d_bf + (size_t)k * wlen;
            }
        }
        base.wlen = wlen;
        // chosen mode: the TT slots (00 family) and the ++ / -- slots (22 family) of a set, each
        // kind with at least mma_min_slots slots, go to the tensor-core kernels, up to kMmaMaxSlots
        // windows per launch; the rest go to the CUDA-core kernels in groups of up to 8
        std::vector<Slot> mma00, mma22;
        if (mode == PS_MODE_CHOSEN && c->tensor_cores)
            for (int k = 0; k < K; ++k)
                for (int s = 0; s < 4; ++s)
                    if ((cases & (1u << s)) && dM[4 * k + s] && s != PS_SPIN_02)
                        (s == PS_SPIN_00 ? mma00 : mma22).push_back(Slot{k, s});
        if ((int)mma00.size() < mma_min_slots(true, lmax)) mma00.clear();
        if ((int)mma22.size() < mma_min_slots(false, lmax)) mma22.clear();
        const int gs = ps::kMaxWin;  // one generation of the families serves up to 8 slots
        const auto groups = group_slots(cases, K, gs, [&](int k, int s) {
            if (!dM[4 * k + s]) return false;
            if (s == PS_SPIN_00) return mma00.empty();
            return s == PS_SPIN_02 || mma22.empty();
        });
        PS_CUDA(c, cudaEventRecord(c->ev0, c->stream));
        if (!mma00.empty() || !mma22.empty()) {
            if ((st = ensure_mtiles(c, lmin, lmax))) return st;
            if ((st = arm_status(c, c->stream))) return st;
        }
        for (const std::vector<Slot>* list : {&mma00, &mma22}) {
            for (size_t i0 = 0; i0 < list->size(); i0 += ps::kMmaMaxSlots) {
                ps::MmaParams mp;
                memset(&mp, 0, sizeof(mp));
                mp.lmin = lmin;
                mp.lmax = lmax;
                mp.nslot = (int)std::min(list->size() - i0, (size_t)ps::kMmaMaxSlots);
                for (int i = 0; i < mp.nslot; ++i) {
                    const Slot q = (*list)[i0 + i];
                    mp.bf[i] = descs[q.k].bf;
                    mp.wW[i] = descs[q.k].wW;
                    mp.parity[i] = q.s == PS_SPIN_00 ? ps::PAR_ALL : (q.s == PS_SPIN_PP ? ps::PAR_EVEN : ps::PAR_ODD);
                    mp.out[i] = dM[4 * q.k + q.s];
                    mp.stage_rows |= host_resident(mp.out[i]);
                }
                mp.ldo = ldm;
                mp.wlen = wlen;
                mp.epilogue = ps::EPI_MCM;
                mp.tiles = c->d_mtiles;
                mp.ntiles = c->nmtiles;
                mp.status = c->d_status;
                mp.tab = c->d_btab;
                PS_CUDA(c, ps::launch_mma(mp, list == &mma00, c->stream));
                c->launches += 2;
            }
        }
        for (size_t g = 0; g < groups.size(); ++g) {
            const auto& grp = groups[g];
            ps::CouplingParams p = base;
            p.nwin = (int)grp.size();
            for (size_t i = 0; i < grp.size(); ++i) {
                p.win[i] = descs[grp[i].k];
                spin_window(grp[i].s, &p.win[i].product, &p.win[i].parity);
                p.out[i] = dM[4 * grp[i].k + grp[i].s];
            }
            p.ldo = ldm;
            if ((st = run_coupling(c, p, mode, false, false))) return st;
        }
        PS_CUDA(c, cudaEventRecord(c->ev1, c->stream));
        c->timed = true;
    }
    return PS_OK;
}

int ps_mcm_set(ps_ctx* c, unsigned cases, const double* const* W, int K, int64_t nW, int lmin, int lmax, int mode,
               double* const* M, int64_t ldm)
{
    int st = check_grid(c, lmin, lmax, nW, ldm);
    if (st) return st;
    if ((st = check_mode(c, mode))) return st;
    if (cases == 0 || (cases & ~0xFu)) return set_err(c, PS_ERR_ARG, "cases mask 0x%x must select bits 0..3", cases);
    if (K < 1 || !W || !M) return set_err(c, PS_ERR_ARG, "K >= 1 and W, M arrays required");
    int nused = 0;
    for (int k = 0; k < K; ++k) {
        if (!W[k]) return set_err(c, PS_ERR_ARG, "W[%d] is NULL", k);
        for (int s = 0; s < 4; ++s) nused += (cases & (1u << s)) && M[4 * k + s];
    }
    if (nused == 0) return set_err(c, PS_ERR_ARG, "every selected output M[4k+s] is NULL");
    PS_CUDA(c, cudaSetDevice(c->device));
    // spectra in: only the entries the families can reach (l3 <= 2 lmax)
    const long long nuse = nW < (int64_t)(2 * lmax + 1) ? nW : (int64_t)(2 * lmax + 1);
    if ((st = ensure(c, &c->d_raw, &c->raw_cap, (size_t)K * nuse))) return st;
    std::vector<const double*> dW(K);
    for (int k = 0; k < K; ++k) {
        PS_CUDA(c, cudaMemcpyAsync(c->d_raw + (size_t)k * nuse, W[k], (size_t)nuse * sizeof(double),
                                   cudaMemcpyHostToDevice, c->stream));
        dW[k] = c->d_raw + (size_t)k * nuse;
    }
    // matrices out: page-locked ones are written in place, the others staged (same leading dimension)
    const size_t n = (size_t)(lmax - lmin + 1);
    std::vector<double*> dM(4 * (size_t)K, nullptr);
    std::vector<int> staged;
    for (int i = 0; i < 4 * K; ++i) {
        if (!(cases & (1u << (i & 3))) || !M[i]) continue;
        if (!(dM[i] = mapped_host(M[i]))) staged.push_back(i);
    }
    if (!staged.empty()) {
        if ((st = ensure(c, &c->d_out, &c->out_cap, staged.size() * n * (size_t)ldm))) return st;
        for (size_t q = 0; q < staged.size(); ++q) dM[staged[q]] = c->d_out + q * n * (size_t)ldm;
    }
    if ((st = ps_mcm_set_device(c, cases, dW.data(), K, nuse, lmin, lmax, mode, dM.data(), ldm))) return st;
    for (int i : staged)
        PS_CUDA(c, cudaMemcpy2DAsync(M[i], (size_t)ldm * sizeof(double), dM[i], (size_t)ldm * sizeof(double),
                                     n * sizeof(double), n, cudaMemcpyDeviceToHost, c->stream));
    PS_CUDA(c, cudaStreamSynchronize(c->stream));
    return check_status(c);
}

int ps_batch_prepare(ps_ctx* c, const ps_problem* probs, int nprob, int gs, int bps)
{
    if (!c) return PS_ERR_ARG;
    if (!probs || nprob < 1) return set_err(c, PS_ERR_ARG, "need at least one problem");
    int st;
    for (int i = 0; i < nprob; ++i)
        if ((st = check_problem(c, probs[i], i))) return st;
    if (gs == 0) gs = c->tuned_group_slots ? c->tuned_group_slots : 4;
    if (gs != 2 && gs != 4 && gs != 8) return set_err(c, PS_ERR_ARG, "group_slots must be 2, 4 or 8 (got %d)", gs);
    PS_CUDA(c, cudaSetDevice(c->device));
    batch_release(c);
    ps_ctx::Batch& b = c->batch;
    // window rows
    std::vector<size_t> row0(nprob);
    size_t rows = 0;
    int max_wlen = 0;
    for (int i = 0; i < nprob; ++i) {
        row0[i] = rows;
        int wlen = 2 * probs[i].lmax + 2;
        rows += (size_t)probs[i].K * wlen;
        max_wlen = std::max(max_wlen, wlen);
    }
    cudaError_t e = cudaMalloc((void**)&b.d_win, rows * sizeof(double));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b.d_bf, rows * sizeof(int2));
    if (e == cudaSuccess) e = cudaMalloc((void**)&b.d_counter, sizeof(unsigned));
    if (e != cudaSuccess) {
        cudaGetLastError();
        batch_release(c);
        return set_err(c, PS_ERR_OOM, "batch buffers: %s", cudaGetErrorString(e));
    }
    std::vector<ps::WinPrep> preps;
    std::vector<ps::CouplingParams> groups;
    std::vector<int4> items;
    std::vector<float> cost;
    std::vector<int2> mtiles, one_mt;
    std::vector<std::pair<long long, int2>> mtile_of;  // (lmin, lmax) key -> (offset in mtiles, count)
    std::vector<size_t> mma_tile_off;                   // per tensor-core launch
    for (int i = 0; i < nprob; ++i) {
        const ps_problem& P = probs[i];
        int wlen = 2 * P.lmax + 2;
        long long nuse = P.nW < (int64_t)(2 * P.lmax + 1) ? P.nW : (int64_t)(2 * P.lmax + 1);
        std::vector<ps::WinDesc> descs(P.K);
        for (int k = 0; k < P.K; ++k) {
            ps::WinPrep w;
            w.src = P.W[k];
            w.nW = nuse;
            w.wW = b.d_win + row0[i] + (size_t)k * wlen;
            w.bf = b.d_bf + row0[i] + (size_t)k * wlen;
            w.wlen = wlen;
            preps.push_back(w);
            descs[k].wW = w.wW;
            descs[k].bf = w.bf;
        }
        // the problem's TT slots and its ++/-- slots, each kind on its own, go to the
        // tensor-core kernels when there are enough of them (as in ps_mcm_set_device)
        unsigned cases_cc = P.cases;
        std::vector<Slot> m00, m22;
        if (c->tensor_cores) {
            for (int k = 0; k < P.K; ++k)
                for (int s = 0; s < 4; ++s)
                    if ((P.cases & (1u << s)) && s != PS_SPIN_02) (s == PS_SPIN_00 ? m00 : m22).push_back(Slot{k, s});
            if ((int)m00.size() >= mma_min_slots(true, P.lmax)) cases_cc &= ~(1u << PS_SPIN_00);
            else m00.clear();
            if ((int)m22.size() >= mma_min_slots(false, P.lmax)) cases_cc &= ~((1u << PS_SPIN_PP) | (1u << PS_SPIN_MM));
            else m22.clear();
        }
        if (!m00.empty() || !m22.empty()) {
            const long long key = ((long long)P.lmin << 32) | (unsigned)P.lmax;
            int2 oc = make_int2(-1, 0);
            for (const auto& t : mtile_of)
                if (t.first == key) oc = t.second;
            if (oc.x < 0) {
                ps::mma_tile_list(P.lmin, P.lmax, one_mt);
                oc = make_int2((int)mtiles.size(), (int)one_mt.size());
                mtiles.insert(mtiles.end(), one_mt.begin(), one_mt.end());
                mtile_of.push_back({key, oc});
            }
            for (const std::vector<Slot>* list : {&m00, &m22}) {
                for (size_t i0 = 0; i0 < list->size(); i0 += ps::kMmaMaxSlots) {
                    ps::MmaParams mp;
                    memset(&mp, 0, sizeof(mp));
                    mp.lmin = P.lmin;
                    mp.lmax = P.lmax;
                    mp.nslot = (int)std::min(list->size() - i0, (size_t)ps::kMmaMaxSlots);
                    for (int q = 0; q < mp.nslot; ++q) {
                        const Slot sl = (*list)[i0 + q];
                        mp.bf[q] = descs[sl.k].bf;
                        mp.wW[q] = descs[sl.k].wW;
                        mp.parity[q] = sl.s == PS_SPIN_00 ? ps::PAR_ALL : (sl.s == PS_SPIN_PP ? ps::PAR_EVEN : ps::PAR_ODD);
                        mp.out[q] = P.M[4 * sl.k + sl.s];
                        mp.stage_rows |= host_resident(mp.out[q]);
                    }
                    mp.ldo = P.ldm;
                    mp.wlen = wlen;
                    mp.epilogue = ps::EPI_MCM;
                    mp.ntiles = oc.y;
                    b.host_mma.push_back(mp);
                    b.host_mma00.push_back(list == &m00);
                    mma_tile_off.push_back((size_t)oc.x);
                }
            }
        }
        if (!cases_cc) continue;
        for (const auto& grp : batch_group_slots(cases_cc, P.K, gs)) {
            ps::CouplingParams g;
            memset(&g, 0, sizeof(g));
            g.lmin = P.lmin;
            g.lmax = P.lmax;
            g.epilogue = ps::EPI_MCM;
            g.nwin = (int)grp.size();
            g.wlen = wlen;
            g.ldo = P.ldm;
            bool f00 = false, f22 = false;
            for (size_t q = 0; q < grp.size(); ++q) {
                g.win[q] = descs[grp[q].k];
                spin_window(grp[q].s, &g.win[q].product, &g.win[q].parity);
                g.out[q] = P.M[4 * grp[q].k + grp[q].s];
                if (g.win[q].product != ps::PROD_22_22) f00 = true;
                if (g.win[q].product != ps::PROD_00_00) f22 = true;
            }
            const int fam = (f00 ? 1 : 0) | (f22 ? 2 : 0);
            const int tmpl = ps::chosen_batch_template(g, gs);
            if (tmpl == 0) {
                batch_release(c);
                return set_err(c, PS_ERR_UNSUPPORTED, "problem %d: no batched kernel body for a window group", i);
            }
            const int gid = (int)groups.size();
            groups.push_back(g);
            // items: up to 8 warp tasks (256 consecutive l2) of one row
            for (int l1 = P.lmin; l1 <= P.lmax; ++l1) {
                for (int l2 = l1; l2 <= P.lmax; l2 += 256) {
                    int ntask = std::min(8, (P.lmax - l2) / 32 + 1);
                    items.push_back(make_int4(gid, l1, l2, ntask | (fam << 8) | (tmpl << 12)));
                    cost.push_back((float)ntask * (2.0f * l1 + 1.0f) * (f22 ? 1.0f : 0.5f));
                }
            }
        }
    }
    // items of one kernel body together (warps of an SM then share their
    // instruction stream), longest first within each body
    std::vector<int> order(items.size());
    for (size_t i = 0; i < order.size(); ++i) order[i] = (int)i;
    std::stable_sort(order.begin(), order.end(), [&](int a, int bb) {
        const int ta = items[a].w >> 8, tb = items[bb].w >> 8;  // template and families
        if (ta != tb) return ta < tb;
        return cost[a] > cost[bb];
    });
    std::vector<int4> sorted(items.size());
    for (size_t i = 0; i < order.size(); ++i) sorted[i] = items[order[i]];
    // the chosen kernel's tiled task lists of every distinct (lmin, lmax), for the launch form
    std::vector<int2> tasks, one;
    std::vector<std::pair<long long, std::pair<size_t, int>>> task_of;  // (lmin, lmax) key -> (offset, count)
    for (int i = 0; i < nprob; ++i) {
        const long long key = ((long long)probs[i].lmin << 32) | (unsigned)probs[i].lmax;
        bool have = false;
        for (const auto& t : task_of) have = have || t.first == key;
        if (have) continue;
        const size_t off = tasks.size();
        tile_task_list(probs[i].lmin, probs[i].lmax, one);
        tasks.insert(tasks.end(), one.begin(), one.end());
        task_of.push_back({key, {off, (int)(tasks.size() - off)}});
    }
    if ((st = dev_upload(c, &b.d_groups, groups)) || (st = dev_upload(c, &b.d_items, sorted)) ||
        (st = dev_upload(c, &b.d_preps, preps)) || (st = dev_upload(c, &b.d_tasks, tasks)) ||
        (st = dev_upload(c, &b.d_mtiles, mtiles))) {
        batch_release(c);
        return st;
    }
    if (!b.host_mma.empty() && (st = alloc_status(c))) {
        batch_release(c);
        return st;
    }
    if (!b.host_mma.empty()) {  // one table for the launches in turn: the size of the largest lmax
        int tab_lmax = 0;
        for (const auto& mp : b.host_mma) tab_lmax = std::max(tab_lmax, mp.lmax);
        size_t cap = 0;
        if ((st = ensure_bytes(c, &b.d_btab, &cap, ps::mma_table_bytes(tab_lmax)))) {
            batch_release(c);
            return st;
        }
    }
    for (size_t m = 0; m < b.host_mma.size(); ++m) {
        b.host_mma[m].tiles = b.d_mtiles + mma_tile_off[m];
        b.host_mma[m].status = c->d_status;
        b.host_mma[m].tab = b.d_btab;
    }
    b.host_groups = groups;
    for (auto& g : b.host_groups) {
        const long long key = ((long long)g.lmin << 32) | (unsigned)g.lmax;
        for (const auto& t : task_of)
            if (t.first == key) {
                g.tasks = b.d_tasks + t.second.first;
                g.ntasks = t.second.second;
            }
    }
    PS_CUDA(c, cudaStreamSynchronize(c->stream));
    int nsm = 0;
    PS_CUDA(c, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    int occ = ps::batch_blocks_per_sm(gs);
    if (bps == 0) bps = c->tuned_blocks_per_sm ? c->tuned_blocks_per_sm : occ;
    b.launches = bps < 0;
    if (!b.launches && (bps < 1 || bps > occ)) bps = occ;
    b.nitems = (int)sorted.size();
    b.npreps = (int)preps.size();
    b.max_wlen = max_wlen;
    b.group_slots = gs;
    b.blocks = b.launches ? 0 : nsm * bps;
    b.ready = true;
    return PS_OK;
}

// The batch's kernels on stream s: window preparation, the tensor-core launches, then the
// CUDA-core part (the persistent kernel, or one launch per group).  The status word of the
// tensor-core launches is cleared by the caller, outside any graph.
static int batch_enqueue(ps_ctx* c, cudaStream_t s)
{
    ps_ctx::Batch& b = c->batch;
    PS_CUDA(c, ps::launch_prep_windows(b.d_preps, b.npreps, b.max_wlen, s));
    if (!b.launches && b.nitems > 0) PS_CUDA(c, cudaMemsetAsync(b.d_counter, 0, sizeof(unsigned), s));
    PS_CUDA(c, cudaEventRecord(c->ev0, s));
    for (size_t m = 0; m < b.host_mma.size(); ++m) PS_CUDA(c, ps::launch_mma(b.host_mma[m], b.host_mma00[m] != 0, s));
    if (b.launches) {  // one chosen-kernel launch per window group, all on the stream
        for (const auto& g : b.host_groups) PS_CUDA(c, ps::launch_chosen(g, s));
    } else if (b.nitems > 0) {
        ps::BatchParams bp;
        bp.groups = b.d_groups;
        bp.items = b.d_items;
        bp.nitems = b.nitems;
        bp.counter = b.d_counter;
        PS_CUDA(c, ps::launch_batch_chosen(bp, b.blocks, b.group_slots, s));
    }
    PS_CUDA(c, cudaEventRecord(c->ev1, s));
    return PS_OK;
}

// kernels one run of the batch launches (window preparation included)
static size_t batch_kernel_count(const ps_ctx::Batch& b)
{
    return 1 + 2 * b.host_mma.size() + (b.launches ? b.host_groups.size() : (b.nitems > 0 ? 1 : 0));
}

int ps_batch_run(ps_ctx* c)
{
    if (!c) return PS_ERR_ARG;
    if (!c->batch.ready) return set_err(c, PS_ERR_ARG, "ps_batch_prepare has not been called");
    PS_CUDA(c, cudaSetDevice(c->device));
    int st;
    if (!c->batch.host_mma.empty() && (st = arm_status(c, c->stream))) return st;
    if ((st = batch_enqueue(c, c->stream))) return st;
    c->launches += batch_kernel_count(c->batch);
    c->timed = true;
    return PS_OK;
}

int ps_batch_graph_launch(ps_ctx* c)
{
    if (!c) return PS_ERR_ARG;
    ps_ctx::Batch& b = c->batch;
    if (!b.ready) return set_err(c, PS_ERR_ARG, "ps_batch_prepare has not been called");
    PS_CUDA(c, cudaSetDevice(c->device));
    if (!b.exec) {
        // capture on the context's own stream (a capturable, non-default stream)
        PS_CUDA(c, cudaStreamSynchronize(c->stream));
        PS_CUDA(c, cudaStreamBeginCapture(c->own_stream, cudaStreamCaptureModeThreadLocal));
        int st = batch_enqueue(c, c->own_stream);
        cudaGraph_t g = nullptr;
        cudaError_t e = cudaStreamEndCapture(c->own_stream, &g);
        if (st) {
            if (g) cudaGraphDestroy(g);
            return st;
        }
        if (e != cudaSuccess) return set_err(c, PS_ERR_CUDA, "graph capture failed: %s", cudaGetErrorString(e));
        e = cudaGraphInstantiate(&b.exec, g, 0);
        cudaGraphDestroy(g);
        if (e != cudaSuccess) {
            b.exec = nullptr;
            return set_err(c, PS_ERR_CUDA, "graph instantiation failed: %s", cudaGetErrorString(e));
        }
    }
    if (!b.host_mma.empty()) {
        int st = arm_status(c, c->stream);
        if (st) return st;
    }
    PS_CUDA(c, cudaGraphLaunch(b.exec, c->stream));
    c->launches += batch_kernel_count(b);
    c->timed = true;
    return PS_OK;
}

int ps_batch_autotune(ps_ctx* c, const ps_problem* probs, int nprob, int* best_gs, int* best_bps, double* best_ms)
{
    if (!c) return PS_ERR_ARG;
    const int cand_gs[3] = {2, 4, 8};
    double best = 1e300;
    int bg = 4, bb = 0, st;
    for (int gi = 0; gi < 3; ++gi) {
        int occ = ps::batch_blocks_per_sm(cand_gs[gi]);
        for (int bps = -1; bps <= occ; ++bps) {  // -1: one launch per group
            if (bps == 0) continue;
            if ((st = ps_batch_prepare(c, probs, nprob, cand_gs[gi], bps))) return st;
            if ((st = ps_batch_run(c))) return st;  // warm-up
            if ((st = ps_batch_run(c))) return st;
            PS_CUDA(c, cudaEventSynchronize(c->ev1));
            float ms = 0.f;
            PS_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
            if (ms < best) {
                best = ms;
                bg = cand_gs[gi];
                bb = bps;
            }
        }
    }
    c->tuned_group_slots = bg;
    c->tuned_blocks_per_sm = bb;
    batch_release(c);
    if (best_gs) *best_gs = bg;
    if (best_bps) *best_bps = bb;
    if (best_ms) *best_ms = best;
    return PS_OK;
}

int ps_decouple_covmat(ps_ctx* c, const double* Y, const double* B1, const double* B2, int64_t n, int64_t ld,
                       double* out, int64_t ldout)
{
    if (!c) return PS_ERR_ARG;
    if (!Y || !B1 || !B2 || !out) return set_err(c, PS_ERR_ARG, "Y, B1, B2 and out must not be NULL");
    if (n < 1 || n > 65535 || ld < n || ldout < n) return set_err(c, PS_ERR_ARG, "need 1 <= n <= 65535, ld >= n");
    PS_CUDA(c, cudaSetDevice(c->device));
    if (!c->la) c->la = ps_linalg_new();
    int st = ps_linalg_decouple(c->la, Y, B1, B2, (int)n, ld, out, ldout, c->stream, c->err, sizeof(c->err), false);
    if (!st) c->launches += 6;
    return st;
}

int ps_decouple_covmat_device(ps_ctx* c, const double* dY, const double* dB1, const double* dB2, int64_t n, int64_t ld,
                              double* dout, int64_t ldout)
{
    if (!c) return PS_ERR_ARG;
    if (!dY || !dB1 || !dB2 || !dout) return set_err(c, PS_ERR_ARG, "Y, B1, B2 and out must not be NULL");
    if (n < 1 || n > 65535 || ld < n || ldout < n) return set_err(c, PS_ERR_ARG, "need 1 <= n <= 65535, ld >= n");
    PS_CUDA(c, cudaSetDevice(c->device));
    if (!c->la) c->la = ps_linalg_new();
    int st = ps_linalg_decouple(c->la, dY, dB1, dB2, (int)n, ld, dout, ldout, c->stream, c->err, sizeof(c->err), true);
    if (!st) c->launches += 6;
    return st;
}

int ps_solve(ps_ctx* c, const double* M, int64_t n, int64_t ldm, const double* b, int nrhs, int64_t ldb, double* x,
             int64_t ldx)
{
    if (!c) return PS_ERR_ARG;
    if (!M || !b || !x) return set_err(c, PS_ERR_ARG, "M, b and x must not be NULL");
    if (n < 1 || n > 65535 || nrhs < 1 || ldm < n || ldb < n || ldx < n)
        return set_err(c, PS_ERR_ARG, "need 1 <= n <= 65535, nrhs >= 1, leading dimensions >= n");
    PS_CUDA(c, cudaSetDevice(c->device));
    if (!c->la) c->la = ps_linalg_new();
    int st = ps_linalg_solve(c->la, M, (int)n, ldm, b, nrhs, ldb, x, ldx, c->stream, c->err, sizeof(c->err));
    if (!st) c->launches += 2;
    return st;
}

// The Xi kernel of either arithmetic on a device W (nW entries) into c->d_out.
static int quickpol_run(ps_ctx* c, const double* dW, long long nW, int lmax, int bl, int bu, int nu1, int nu2, int s1,
                        int s2, int mode)
{
    const size_t n = (size_t)lmax + 1;
    if (mode == PS_MODE_CHOSEN) {
        const size_t nf = (size_t)nW / 2 + 2;  // nW floats, then one int
        int st = ensure(c, &c->d_qp, &c->qp_cap, nf + 1);
        if (st) return st;
        PS_CUDA(c, ps::launch_quickpol_ff(dW, nW, lmax, bl, bu, nu1, nu2, s1, s2, c->d_out, (long long)n,
                                          (float*)c->d_qp, (int*)(c->d_qp + nf), c->stream));
        c->launches += 2;
    } else {
        PS_CUDA(c, ps::launch_quickpol(dW, nW, lmax, bl, bu, nu1, nu2, s1, s2, c->d_out, (long long)n, c->stream));
        c->launches++;
    }
    return PS_OK;
}

int ps_quickpol_xi(ps_ctx* c, int nu1, int nu2, int s1, int s2, const double* W, int64_t nW, int lmax, int bl, int bu,
                   int mode, double* Xi, int64_t ldx)
{
    if (!c) return PS_ERR_ARG;
    if (!W || !Xi) return set_err(c, PS_ERR_ARG, "W and Xi must not be NULL");
    if (lmax < 0 || lmax > PS_MAX_LMAX || nW < 1 || bl < 0 || bu < 0 || ldx < (int64_t)lmax + 1)
        return set_err(c, PS_ERR_ARG, "need 0 <= lmax <= %d, nW >= 1, bandwidths >= 0, ldx >= lmax+1", PS_MAX_LMAX);
    if (abs(nu1) > 64 || abs(nu2) > 64 || abs(s1) > 64 || abs(s2) > 64)
        return set_err(c, PS_ERR_ARG, "spins beyond +-64 are not supported");
    if (mode != PS_MODE_PLAIN_FP64 && mode != PS_MODE_CHOSEN) return set_err(c, PS_ERR_ARG, "unknown mode %d", mode);
    PS_CUDA(c, cudaSetDevice(c->device));
    const size_t n = (size_t)lmax + 1;
    const long long nuse = nW < (int64_t)(2 * lmax + 1) ? nW : (int64_t)(2 * lmax + 1);
    int st;
    if ((st = ensure(c, &c->d_raw, &c->raw_cap, (size_t)nuse))) return st;
    if ((st = ensure(c, &c->d_out, &c->out_cap, n * n))) return st;
    PS_CUDA(c, cudaMemcpyAsync(c->d_raw, W, (size_t)nuse * sizeof(double), cudaMemcpyHostToDevice, c->stream));
    PS_CUDA(c, cudaMemsetAsync(c->d_out, 0, n * n * sizeof(double), c->stream));
    PS_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    if ((st = quickpol_run(c, c->d_raw, nuse, lmax, bl, bu, nu1, nu2, s1, s2, mode))) return st;
    PS_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    c->timed = true;
    PS_CUDA(c, cudaMemcpy2DAsync(Xi, (size_t)ldx * sizeof(double), c->d_out, n * sizeof(double), n * sizeof(double), n,
                                 cudaMemcpyDeviceToHost, c->stream));
    PS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PS_OK;
}

// Shared by ps_window_W and ps_window_W_device: dA/dB are device sets (null = zeros).
static int window_run(ps_ctx* c, const double* const* dA, const double* const* dB, int nterms, int lmax, int mmax,
                      int lout, double* dW, bool per_l = true)
{
    ps::AlmParams p = {};
    p.nterms = nterms;
    p.lmax = lmax;
    p.mmax = mmax;
    p.lout = lout;
    p.mchunk = ps::kAlmChunk;
    p.nmchunks = ps::alm2cl_chunks(mmax);
    for (int t = 0; t < nterms; ++t) {
        p.a[t] = (const double2*)dA[t];
        p.b[t] = (const double2*)dB[t];
    }
    int st = ensure(c, &c->d_part, &c->part_cap, (size_t)nterms * p.nmchunks * ((size_t)lout + 1));
    if (st) return st;
    p.partial = c->d_part;
    // the context's kernel time is the partial-sum kernel's (the reduction is small)
    PS_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    PS_CUDA(c, ps::launch_alm2cl(p, 1.0 / nterms, per_l, dW, c->stream, c->ev1));
    c->launches += 2;
    c->timed = true;
    return PS_OK;
}

static int window_check(ps_ctx* c, const double* const* A, const double* const* B, int nterms, int lmax, int mmax,
                        int lout, const double* W)
{
    if (!A || !B || !W) return set_err(c, PS_ERR_ARG, "A, B and W must not be NULL");
    if (nterms < 1 || nterms > ps::kAlmMaxTerms)
        return set_err(c, PS_ERR_ARG, "need 1 <= nterms <= %d, got %d", ps::kAlmMaxTerms, nterms);
    if (lmax < 0 || lmax > 65535 || mmax < 0 || mmax > lmax || lout < 0 || lout > lmax)
        return set_err(c, PS_ERR_ARG, "need 0 <= mmax <= lmax <= 65535 and 0 <= lout <= lmax");
    return PS_OK;
}

int ps_window_W_device(ps_ctx* c, const double* const* dA, const double* const* dB, int nterms, int lmax, int mmax,
                       int lout, double* dW)
{
    if (!c) return PS_ERR_ARG;
    int st = window_check(c, dA, dB, nterms, lmax, mmax, lout, dW);
    if (st) return st;
    for (int t = 0; t < nterms; ++t)
        if (((uintptr_t)dA[t] | (uintptr_t)dB[t]) & 15)
            return set_err(c, PS_ERR_ARG, "coefficient set %d is not 16-byte aligned", t);
    PS_CUDA(c, cudaSetDevice(c->device));
    return window_run(c, dA, dB, nterms, lmax, mmax, lout, dW);
}

int ps_window_W(ps_ctx* c, const double* const* A, const double* const* B, int nterms, int lmax, int mmax, int lout,
                double* W)
{
    if (!c) return PS_ERR_ARG;
    int st = window_check(c, A, B, nterms, lmax, mmax, lout, W);
    if (st) return st;
    PS_CUDA(c, cudaSetDevice(c->device));
    // copy each distinct host set once (an auto-spectrum term names the same set twice)
    const size_t nalm = (size_t)(mmax + 1) * (mmax + 2) / 2 + (size_t)(mmax + 1) * (lmax - mmax);
    std::vector<const double*> uniq;
    for (int t = 0; t < nterms; ++t)
        for (const double* q : {A[t], B[t]})
            if (q && std::find(uniq.begin(), uniq.end(), q) == uniq.end()) uniq.push_back(q);
    // A page-locked, mapped set is read by the kernel where it lies (over the
    // host link, once); any other set is copied to the device first.
    std::vector<const double*> where(uniq.size());
    size_t ncopy = 0;
    for (size_t u = 0; u < uniq.size(); ++u) {
        const double* m = mapped_host(const_cast<double*>(uniq[u]));
        where[u] = (m && ((uintptr_t)m & 15) == 0) ? m : nullptr;
        if (!where[u]) ++ncopy;
    }
    if ((st = ensure(c, &c->d_alm, &c->alm_cap, 2 * nalm * (ncopy ? ncopy : 1)))) return st;
    if ((st = ensure(c, &c->d_out, &c->out_cap, (size_t)lout + 1))) return st;
    for (size_t u = 0, k = 0; u < uniq.size(); ++u) {
        if (where[u]) continue;
        where[u] = c->d_alm + 2 * nalm * k++;
        PS_CUDA(c, cudaMemcpyAsync(const_cast<double*>(where[u]), uniq[u], 2 * nalm * sizeof(double),
                                   cudaMemcpyHostToDevice, c->stream));
    }
    auto dev = [&](const double* q) -> const double* {
        if (!q) return nullptr;
        return where[(size_t)(std::find(uniq.begin(), uniq.end(), q) - uniq.begin())];
    };
    const double* dA[ps::kAlmMaxTerms];
    const double* dB[ps::kAlmMaxTerms];
    for (int t = 0; t < nterms; ++t) {
        dA[t] = dev(A[t]);
        dB[t] = dev(B[t]);
    }
    if ((st = window_run(c, dA, dB, nterms, lmax, mmax, lout, c->d_out))) return st;
    PS_CUDA(c, cudaMemcpyAsync(W, c->d_out, ((size_t)lout + 1) * sizeof(double), cudaMemcpyDeviceToHost, c->stream));
    PS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PS_OK;
}

int ps_quickpol_xi_alm(ps_ctx* c, int nu1, int nu2, int s1, int s2, const double* omega1, const double* omega2,
                       int alm_lmax, int alm_mmax, int lmax, int bl, int bu, int mode, double* Xi, int64_t ldx)
{
    if (!c) return PS_ERR_ARG;
    if (!omega1 || !omega2 || !Xi) return set_err(c, PS_ERR_ARG, "omega1, omega2 and Xi must not be NULL");
    if (alm_lmax < 0 || alm_lmax > 65535 || alm_mmax < 0 || alm_mmax > alm_lmax)
        return set_err(c, PS_ERR_ARG, "need 0 <= alm_mmax <= alm_lmax <= 65535");
    if (lmax < 0 || lmax > PS_MAX_LMAX || bl < 0 || bu < 0 || ldx < (int64_t)lmax + 1)
        return set_err(c, PS_ERR_ARG, "need 0 <= lmax <= %d, bandwidths >= 0, ldx >= lmax+1", PS_MAX_LMAX);
    if (abs(nu1) > 64 || abs(nu2) > 64 || abs(s1) > 64 || abs(s2) > 64)
        return set_err(c, PS_ERR_ARG, "spins beyond +-64 are not supported");
    if (mode != PS_MODE_PLAIN_FP64 && mode != PS_MODE_CHOSEN) return set_err(c, PS_ERR_ARG, "unknown mode %d", mode);
    PS_CUDA(c, cudaSetDevice(c->device));
    // Xi reads W[l'] only for l' <= l + l'' <= 2 lmax, so only the coefficients
    // with l <= lw enter; those rows are packed into a smaller set (lmax lw) on
    // the host before the copy when the given sets reach further.
    const int lw = std::min(alm_lmax, 2 * lmax);
    const int mw = std::min(alm_mmax, lw);
    const size_t nalm = (size_t)(mw + 1) * (mw + 2) / 2 + (size_t)(mw + 1) * (lw - mw);
    const bool same = omega1 == omega2;
    int st;
    if ((st = ensure(c, &c->d_alm, &c->alm_cap, 2 * nalm * (same ? 1 : 2)))) return st;
    if ((st = ensure(c, &c->d_spec, &c->spec_cap, (size_t)lw + 1))) return st;
    const size_t n = (size_t)lmax + 1;
    if ((st = ensure(c, &c->d_out, &c->out_cap, n * n))) return st;
    auto upload = [&](const double* src, double* dst) -> int {
        if (lw == alm_lmax) {
            PS_CUDA(c, cudaMemcpyAsync(dst, src, 2 * nalm * sizeof(double), cudaMemcpyHostToDevice, c->stream));
            return PS_OK;
        }
        PS_CUDA(c, cudaStreamSynchronize(c->stream));  // the pinned staging is reused for the second set
        int st2 = ensure_pinned(c, 2 * nalm);
        if (st2) return st2;
        // rows m: l = m..lw, at m (2 alm_lmax + 1 - m) / 2 + l in the source and
        // m (2 lw + 1 - m) / 2 + l in the packed set; packed by a few host threads
        const int nth = (int)std::min<size_t>(8, 1 + nalm / (1 << 18));
        std::vector<std::thread> pool;
        for (int t = 0; t < nth; ++t)
            pool.emplace_back([&, t] {
                for (int m = t; m <= mw; m += nth) {
                    const size_t from = (size_t)m * (2 * (size_t)alm_lmax + 1 - m) / 2 + m;
                    const size_t to = (size_t)m * (2 * (size_t)lw + 1 - m) / 2 + m;
                    memcpy(c->h_pack + 2 * to, src + 2 * from, 2 * (size_t)(lw - m + 1) * sizeof(double));
                }
            });
        for (auto& th : pool) th.join();
        PS_CUDA(c, cudaMemcpyAsync(dst, c->h_pack, 2 * nalm * sizeof(double), cudaMemcpyHostToDevice, c->stream));
        PS_CUDA(c, cudaStreamSynchronize(c->stream));
        return PS_OK;
    };
    if ((st = upload(omega1, c->d_alm))) return st;
    const double* dA = c->d_alm;
    const double* dB = c->d_alm;
    if (!same) {
        if ((st = upload(omega2, c->d_alm + 2 * nalm))) return st;
        dB = c->d_alm + 2 * nalm;
    }
    // quickpolW on the GPU: sum_m omega1_lm conj(omega2_lm), no 1 / (2l + 1)
    if ((st = window_run(c, &dA, &dB, 1, lw, mw, lw, c->d_spec, false))) return st;
    PS_CUDA(c, cudaMemsetAsync(c->d_out, 0, n * n * sizeof(double), c->stream));
    if ((st = quickpol_run(c, c->d_spec, (long long)lw + 1, lmax, bl, bu, nu1, nu2, s1, s2, mode))) return st;
    PS_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    PS_CUDA(c, cudaMemcpy2DAsync(Xi, (size_t)ldx * sizeof(double), c->d_out, n * sizeof(double), n * sizeof(double), n,
                                 cudaMemcpyDeviceToHost, c->stream));
    PS_CUDA(c, cudaStreamSynchronize(c->stream));
    return PS_OK;
}

int ps_probe_fma_peak(ps_ctx* c, int fp64, double* flops)
{
    if (!c || !flops) return PS_ERR_ARG;
    PS_CUDA(c, cudaSetDevice(c->device));
    int nsm = 0;
    PS_CUDA(c, cudaDeviceGetAttribute(&nsm, cudaDevAttrMultiProcessorCount, c->device));
    int blocks = nsm * 8;
    size_t dummy = 0;
    int st = ensure(c, &c->d_probe, &dummy, (size_t)blocks);
    if (st) return st;
    int iters = fp64 ? 4096 : 262144;
    PS_CUDA(c, ps::launch_fma_probe(fp64, c->d_probe, blocks, 64, c->stream));  // warm-up
    c->launches++;
    PS_CUDA(c, cudaEventRecord(c->ev0, c->stream));
    PS_CUDA(c, ps::launch_fma_probe(fp64, c->d_probe, blocks, iters, c->stream));
    c->launches++;
    PS_CUDA(c, cudaEventRecord(c->ev1, c->stream));
    PS_CUDA(c, cudaEventSynchronize(c->ev1));
    float ms = 0.f;
    PS_CUDA(c, cudaEventElapsedTime(&ms, c->ev0, c->ev1));
    double fl = (double)blocks * 256.0 * (double)iters * 8.0 * 2.0;
    *flops = fl / (ms * 1e-3);
    c->timed = false;
    cudaFree(c->d_probe);
    c->d_probe = nullptr;
    return PS_OK;
}

}  // extern "C"
