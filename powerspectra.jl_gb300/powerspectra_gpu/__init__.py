"""GB300 mode-coupling / covariance hot path of PowerSpectra.jl (host side).

The compute runs in libpowerspectra_gpu.so (CUDA, sm_103a) behind the C ABI of
include/powerspectra_gpu.h; this package is the host-side mirror of the
reference's `mcm` / `coupledcov` entry points and their return types.
"""
from ._lib import (Context, PowerSpectraArgumentError, PowerSpectraGPUError, default_context, load,  # noqa: F401
                   PS_SPIN_00, PS_SPIN_02, PS_SPIN_PP, PS_SPIN_MM, PS_MODE_PLAIN_FP64, PS_MODE_CHOSEN)
from .spectralarray import BlockSpectralMatrix, SpectralArray, SpectralVector, spectralones, spectralzeros  # noqa
from .modecoupling import (inner_mcm00, inner_mcm02, inner_mcmMM, inner_mcmPP, inner_mcmPPMM, mcm)  # noqa: F401
from .covariance import (ConstantDict, WindowWorkspace, coupledcov, loop_covEEEE, loop_covTEEE,  # noqa: F401
                         loop_covTEEE_planck, loop_covTETE, loop_covTTEE, loop_covTTTE, loop_covTTTT)
from .workspace import AlmWindowWorkspace, alm2cl, n_alms, wterms  # noqa: F401
