// ps_chosen8.cu -- the chosen coupling kernel (ps_chosen_task.cuh) for window
// groups of 6-8 slots: one generation of the families per pair serves up to 8
// (window, spin case) slots.
#include "ps_chosen_task.cuh"

namespace ps {

cudaError_t launch_chosen8(const CouplingParams& p, uint32_t spec, bool n00, bool n22, cudaStream_t s)
{
    const int nw = p.nwin;
    if (spec_fits(spec, nw, rep(W00, 8), 8)) return launch_cfg<8, rep(W00, 8)>(p, n00, n22, s);
    if (spec_fits(spec, nw, rep(WPP, 8), 8)) return launch_cfg<8, rep(WPP, 8)>(p, n00, n22, s);
    if (spec_fits(spec, nw, rep(WMM, 8), 8)) return launch_cfg<8, rep(WMM, 8)>(p, n00, n22, s);
    if (spec_fits(spec, nw, rep(W02, 8), 8)) return launch_cfg<8, rep(W02, 8)>(p, n00, n22, s);
    if (spec_fits(spec, nw, S_PPMM4, 8)) return launch_cfg<8, S_PPMM4>(p, n00, n22, s);
    if (spec_fits(spec, nw, S_MCM8, 8)) return launch_cfg<8, S_MCM8>(p, n00, n22, s);
    return launch_cfg<8, 0>(p, n00, n22, s);
}

}  // namespace ps
