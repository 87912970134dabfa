// ps_batch_chosen.cu -- the persistent batched kernel over the chosen
// coupling task (ps_chosen_task.cuh).
#include "ps_chosen_task.cuh"

namespace ps {

// Persistent batched kernel: every warp takes the next item of a work queue
// that spans all problems and window groups of the batch, until the queue is
// empty.  The queue is ordered by kernel body (the group's compile-time slot
// list), then by decreasing family length.  An item is up to 8 warp tasks (256
// consecutive l2) of one row of one window group; each warp copies its
// group's CouplingParams from global into shared memory when the group
// changes.
// The six per-window slot patterns a batch group can hold, as compile-time slot
// lists of NWIN slots (4 or 8): TT, (++, --) pairs, TT/TE/++/--, ++, --, TE.
template <int NWIN>
struct BatchSets;
template <>
struct BatchSets<4> {
    static constexpr uint32_t s[6] = {rep(W00, 4), S_PPMM2, S_MCM4, rep(WPP, 4), rep(WMM, 4), rep(W02, 4)};
};
template <>
struct BatchSets<8> {
    static constexpr uint32_t s[6] = {rep(W00, 8), S_PPMM4, S_MCM8, rep(WPP, 8), rep(WMM, 8), rep(W02, 8)};
};

template <int NWIN>
__global__ void __launch_bounds__(kWarpsPerBlock * 32, NWIN <= 4 ? 5 : 3) k_batch_chosen(const BatchParams bp)
{
    __shared__ __align__(16) float sW[kWarpsPerBlock][2][NWIN][kSlots];  // 16-byte slot reads (4-slot bodies)
    // each warp's copy of its current group's parameters: read in the inner
    // loops, so they live in shared memory rather than behind global loads
    __shared__ CouplingParams sG[kWarpsPerBlock];
    __shared__ int2 sR[kWarpsPerBlock][2][NWIN][kSlots];
    __shared__ CoefTab sT[kWarpsPerBlock];
    const int warp = threadIdx.x >> 5;
    const int lane = threadIdx.x & 31;
    float* sF = &sW[warp][0][0][0];
    float* sB = &sW[warp][1][0][0];
    int cur = -1;
    for (;;) {
        int it = 0;
        if (lane == 0) it = (int)atomicAdd(bp.counter, 1u);
        it = __shfl_sync(0xffffffffu, it, 0);
        if (it >= bp.nitems) break;  // every warp leaves once the queue is drained; nothing waits
        const int4 item = bp.items[it];  // (group, l1, first l2, tasks | families << 8 | template << 12)
        if (item.x != cur) {
            const int* src = reinterpret_cast<const int*>(bp.groups + item.x);
            int* dst = reinterpret_cast<int*>(&sG[warp]);
            for (int q = lane; q < (int)(sizeof(CouplingParams) / sizeof(int)); q += 32) dst[q] = src[q];
            cur = item.x;
            __syncwarp();
        }
        const CouplingParams& g = sG[warp];
        const int ntask = item.w & 0xff, tmpl = item.w >> 12;  // bits 8-11 (families) only order the queue
        for (int q = 0; q < ntask; ++q) {
            const int l2_0 = item.z + 32 * q;
            switch (tmpl) {  // the group's compile-time slot set (prepare never emits others)
            case 1: chosen_task<NWIN, true, false, BatchSets<NWIN>::s[0]>(g, item.y, l2_0, sF, sB, &sR[warp][0][0][0], sT[warp], lane); break;
            case 2: chosen_task<NWIN, false, true, BatchSets<NWIN>::s[1]>(g, item.y, l2_0, sF, sB, &sR[warp][0][0][0], sT[warp], lane); break;
            case 3: chosen_task<NWIN, true, true, BatchSets<NWIN>::s[2]>(g, item.y, l2_0, sF, sB, &sR[warp][0][0][0], sT[warp], lane); break;
            case 4: chosen_task<NWIN, false, true, BatchSets<NWIN>::s[3]>(g, item.y, l2_0, sF, sB, &sR[warp][0][0][0], sT[warp], lane); break;
            case 5: chosen_task<NWIN, false, true, BatchSets<NWIN>::s[4]>(g, item.y, l2_0, sF, sB, &sR[warp][0][0][0], sT[warp], lane); break;
            case 6: chosen_task<NWIN, true, true, BatchSets<NWIN>::s[5]>(g, item.y, l2_0, sF, sB, &sR[warp][0][0][0], sT[warp], lane); break;
            default: break;  // prepare rejects groups without a body
            }
            __syncwarp();
        }
    }
}

cudaError_t launch_batch_chosen(const BatchParams& bp, int blocks, int nwin, cudaStream_t s)
{
    if (bp.nitems <= 0) return cudaSuccess;
    if (nwin > 4)
        k_batch_chosen<8><<<blocks, kWarpsPerBlock * 32, 0, s>>>(bp);
    else
        k_batch_chosen<4><<<blocks, kWarpsPerBlock * 32, 0, s>>>(bp);
    return cudaGetLastError();
}

int batch_blocks_per_sm(int nwin)
{
    int n = 0;
    cudaError_t e = nwin > 4 ? cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_chosen<8>, kWarpsPerBlock * 32, 0)
                             : cudaOccupancyMaxActiveBlocksPerMultiprocessor(&n, k_batch_chosen<4>, kWarpsPerBlock * 32, 0);
    if (e != cudaSuccess) {
        cudaGetLastError();
        return 1;
    }
    return n > 0 ? n : 1;
}

int chosen_batch_template(const CouplingParams& p, int nwin)
{
    const uint32_t spec = spec_of(p);
    const uint32_t* sets = nwin > 4 ? BatchSets<8>::s : BatchSets<4>::s;
    const int n = nwin > 4 ? 8 : 4;
    for (int i = 0; i < 6; ++i)
        if (spec_fits(spec, p.nwin, sets[i], n)) return i + 1;
    return 0;
}

}  // namespace ps
