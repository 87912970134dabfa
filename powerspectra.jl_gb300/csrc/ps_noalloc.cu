// ps_noalloc.cu -- mode-coupling matrices without any device allocation.
//
// Some callers of this library are not allowed to call cudaMalloc: code whose
// device memory is owned by another allocator (a framework's caching pool or a
// fixed budget that must not grow), and pipelines that cannot afford the
// implicit device-wide synchronisation that cudaMalloc and cudaFree may cause
// in the middle of their stream work.  ps_mcm_multi_device_noalloc serves
// them: it runs the chosen coupling kernel (the same kernel ps_mcm_multi_device
// runs with PS_MODE_CHOSEN) with its scratch memory taken from a fixed array
// that lives in the library's device image instead of from cudaMalloc.
//
// The scratch holds the padded windows, their split (mantissa, exponent) copies
// and the warp task list.  Every call rewrites all of it before use, so nothing
// has to start at zero, but every call on a device shares this one array:
// calls whose GPU work overlaps (on different streams or threads) race.
#include "ps_internal.cuh"
#include "ps_tiles.h"

#include <atomic>
#include <stdint.h>
#include <string.h>

namespace {

constexpr int kNoAllocMaxLmax = 4095;  // largest lmax the fixed scratch serves
constexpr int kNoAllocMaxWlen = 2 * kNoAllocMaxLmax + 2;
// The task list is longest for lmin = 0 (n = 4096 rows, 128 column blocks, all
// 1024 row groups); any other range with lmax <= 4095 has at most as many tiles.
constexpr long long kNoAllocMaxTasks = ps_tiles::task_count(0, kNoAllocMaxLmax);
static_assert(kNoAllocMaxTasks == 264192, "4 tasks per tile, 66048 tiles at lmax 4095");

// windows: 4 x wlen doubles, split copies: 4 x wlen int2, tasks: int2 each
constexpr size_t kWinBytes = 4ull * kNoAllocMaxWlen * sizeof(double);
constexpr size_t kBfBytes = 4ull * kNoAllocMaxWlen * sizeof(int2);
constexpr size_t kTaskBytes = (size_t)kNoAllocMaxTasks * sizeof(int2);
constexpr size_t kScratchBytes = kWinBytes + kBfBytes + kTaskBytes;  // 2.6 MB
static_assert(kWinBytes % 256 == 0 && kBfBytes % 256 == 0, "each scratch region starts 256-byte aligned");

static __device__ __align__(256) unsigned char g_scratch[kScratchBytes];

// Device address of g_scratch per device.  It is looked up with the device
// current on every call whose stream is not capturing (cheap, and correct
// again after a device reset reloads the library image); a call made during
// stream capture uses the address the last uncaptured call on that device
// found.  Atomic, so host threads may make their first calls concurrently.
constexpr int kMaxDevices = 64;
static std::atomic<void*> g_scratch_addr[kMaxDevices];

// One thread per row group writes its tiles' tasks (the list of ps_tiles.h).
__global__ void k_fill_tiles(int2* __restrict__ tasks, int lmin, int lmax)
{
    const ps_tiles::Geometry G = ps_tiles::geometry(lmin, lmax);
    for (int g = G.glo + blockIdx.x * blockDim.x + threadIdx.x; g < 8 * G.nb; g += gridDim.x * blockDim.x) {
        long long t = ps_tiles::group_offset(G, g);
        for (int b = g / 8; b < G.nb; ++b)
            for (int q = 0; q < 4; ++q, ++t) {
                const int l1 = G.o + 4 * g + q;
                tasks[t] = make_int2(l1 >= lmin ? l1 : -1, G.o + 32 * b);
            }
    }
}

// The scratch address on the current device `dev`, or nullptr.
void* scratch_address(int dev, cudaStream_t s)
{
    cudaStreamCaptureStatus cs = cudaStreamCaptureStatusNone;
    if (cudaStreamIsCapturing(s, &cs) != cudaSuccess) {
        cudaGetLastError();
        return nullptr;
    }
    if (cs != cudaStreamCaptureStatusNone) return g_scratch_addr[dev].load();
    void* ptr = nullptr;
    if (cudaGetSymbolAddress(&ptr, g_scratch) != cudaSuccess || !ptr) {
        cudaGetLastError();
        return nullptr;
    }
    g_scratch_addr[dev].store(ptr);
    return ptr;
}

}  // namespace

extern "C" int ps_mcm_multi_device_noalloc(unsigned cases, const double* const dW[4], int64_t nW, int lmin, int lmax,
                                           double* const dM[4], int64_t ldm, void* stream)
{
    if (cases == 0 || (cases & ~0xFu) || !dW || !dM) return PS_ERR_ARG;
    if (lmin < 0 || lmax < lmin || nW < 1 || ldm < (int64_t)(lmax - lmin + 1)) return PS_ERR_ARG;
    if (lmax > kNoAllocMaxLmax) return PS_ERR_ARG;  // beyond what the fixed scratch holds
    for (int s = 0; s < 4; ++s)
        if ((cases & (1u << s)) && (!dW[s] || !dM[s])) return PS_ERR_ARG;
    const long long ntasks = ps_tiles::task_count(lmin, lmax);
    if (ntasks > kNoAllocMaxTasks) return PS_ERR_ARG;  // bounded by the static_assert above for lmax <= 4095

    cudaStream_t s = (cudaStream_t)stream;
    int dev = 0, sdev = 0;
    if (cudaGetDevice(&dev) != cudaSuccess || dev < 0 || dev >= kMaxDevices) {
        cudaGetLastError();
        return PS_ERR_CUDA;
    }
    // the scratch lives on the current device: a stream of another device is an argument error
    if (cudaStreamGetDevice(s, &sdev) != cudaSuccess) {
        cudaGetLastError();
        return PS_ERR_ARG;
    }
    if (sdev != dev) return PS_ERR_ARG;
    unsigned char* base = (unsigned char*)scratch_address(dev, s);
    if (!base) return PS_ERR_CUDA;  // no lookup yet on this device (first call made during capture) or CUDA error
    double* win = (double*)base;
    int2* bf = (int2*)(base + kWinBytes);
    int2* tasks = (int2*)(base + kWinBytes + kBfBytes);

    ps::CouplingParams p;
    memset(&p, 0, sizeof(p));
    p.lmin = lmin;
    p.lmax = lmax;
    p.epilogue = ps::EPI_MCM;
    p.wlen = 2 * lmax + 2;
    p.ldo = ldm;
    const long long nuse = nW < (int64_t)(2 * lmax + 1) ? nW : (int64_t)(2 * lmax + 1);
    int K = 0;
    for (int sp = 0; sp < 4; ++sp) {
        if (!(cases & (1u << sp))) continue;
        double* w = win + (size_t)K * p.wlen;
        int2* b = bf + (size_t)K * p.wlen;
        if (ps::launch_pad_windows(w, dW[sp], nuse, p.wlen, s) != cudaSuccess) return PS_ERR_CUDA;
        if (ps::launch_split_windows(b, w, p.wlen, s) != cudaSuccess) return PS_ERR_CUDA;
        p.win[K].wW = w;
        p.win[K].bf = b;
        switch (sp) {
        case PS_SPIN_00: p.win[K].product = ps::PROD_00_00; p.win[K].parity = ps::PAR_ALL; break;
        case PS_SPIN_02: p.win[K].product = ps::PROD_00_22; p.win[K].parity = ps::PAR_EVEN; break;
        case PS_SPIN_PP: p.win[K].product = ps::PROD_22_22; p.win[K].parity = ps::PAR_EVEN; break;
        default: p.win[K].product = ps::PROD_22_22; p.win[K].parity = ps::PAR_ODD; break;
        }
        p.out[K] = dM[sp];
        ++K;
    }
    p.nwin = K;
    const ps_tiles::Geometry G = ps_tiles::geometry(lmin, lmax);
    const int groups = 8 * G.nb - G.glo;
    k_fill_tiles<<<(groups + 255) / 256, 256, 0, s>>>(tasks, lmin, lmax);
    if (cudaGetLastError() != cudaSuccess) return PS_ERR_CUDA;
    p.tasks = tasks;
    p.ntasks = (int)ntasks;
    if (ps::launch_chosen(p, s) != cudaSuccess) return PS_ERR_CUDA;
    return PS_OK;
}
