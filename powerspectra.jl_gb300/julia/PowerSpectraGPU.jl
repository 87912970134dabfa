# PowerSpectraGPU.jl -- ccall shim that routes PowerSpectra.jl's hot loops to
# libpowerspectra_gpu.so (the C ABI in include/powerspectra_gpu.h).
#
# Loading this module after PowerSpectra adds more specific methods for
# Float64 SpectralArrays (any dense column-major storage) to
#     inner_mcm⁰⁰!, inner_mcm⁰²!, inner_mcm⁺⁺!, inner_mcm⁻⁻!   (src/modecoupling.jl:78-159)
#     loop_covTTTT!, loop_covEEEE!, loop_covTTTE!, loop_covTETE!,
#     loop_covTEEE!, loop_covTEEE_planck!, loop_covTTEE!        (src/covariance.jl:92-446)
#     decouple_covmat                                            (src/covariance.jl:8-14)
#     quickpolΞ!                                                 (src/beam.jl:72-109)
#     window_function_W!                                         (src/workspace.jl:174-213)
# so `mcm`, `coupledcov` and `master` keep their signatures and return types
# while the (l1, l2) loops run on the GPU.  There is no CPU fallback: a missing
# library or device raises.
module PowerSpectraGPU

using PowerSpectra
import PowerSpectra: SpectralArray, SpectralVector
import Healpix

const libps = get(ENV, "POWERSPECTRA_GPU_LIB",
                  joinpath(@__DIR__, "..", "lib", "libpowerspectra_gpu.so"))

const PS_SPIN_00 = Cint(0)
const PS_SPIN_02 = Cint(1)
const PS_SPIN_PP = Cint(2)
const PS_SPIN_MM = Cint(3)
const PS_MODE_PLAIN_FP64 = Cint(0)
const PS_MODE_CHOSEN = Cint(1)
const COV = Dict(:TTTT => Cint(0), :EEEE => Cint(1), :TTTE => Cint(2), :TETE => Cint(3),
                 :TEEE => Cint(4), :TEEE_planck => Cint(5), :TTEE => Cint(6))

# Arithmetic used by the overrides.  The default, PS_MODE_PLAIN_FP64, runs the
# recurrences in FP64 and matches the reference's Float64 loops to 1e-12
# relative.  PS_MODE_CHOSEN (FP32-pipe recurrences, <= 1e-6 relative) is
# opt-in: `PowerSpectraGPU.MODE[] = PowerSpectraGPU.PS_MODE_CHOSEN`.
const MODE = Ref(PS_MODE_PLAIN_FP64)
# one library context per Julia thread (a context is not thread-safe)
const CTXS = Dict{Int,Ptr{Cvoid}}()
const CTX_LOCK = ReentrantLock()

function ctx()
    tid = Threads.threadid()
    lock(CTX_LOCK) do
        get!(CTXS, tid) do
            h = Ref{Ptr{Cvoid}}(C_NULL)
            st = ccall((:ps_create, libps), Cint, (Cint, Ref{Ptr{Cvoid}}), Cint(0), h)
            st == 0 || error("powerspectra_gpu: ps_create failed with status $st (no usable CUDA device?)")
            h[]
        end
    end
end

function check(st, c)
    st == 0 && return nothing
    msg = unsafe_string(ccall((:ps_last_error, libps), Cstring, (Ptr{Cvoid},), c))
    st == 1 ? throw(ArgumentError(msg)) : error("powerspectra_gpu error $st: $msg")
end

# Every override takes a SpectralArray{Float64,2} whatever its storage type.
# `mcm` and `coupledcov` allocate with spectralzeros(lmin:lmax, lmin:lmax)
# (src/spectralarray.jl:74), whose parent is an OffsetArray over a Matrix, so a
# signature pinned to a Matrix parent would never be selected and the
# reference's CPU loops would run instead.
const FMat = SpectralArray{Float64,2}

# The innermost array under the SpectralArray / OffsetArray wrappers.
function storage(A)
    P = parent(A)
    return P === A ? A : storage(P)
end

# Column-major memory the library can write for 𝐌 and its leading dimension.
# Dense column-major storage is passed as is; any other storage goes through a
# Matrix that `writeback!` copies into it after the call.
function dense_out(𝐌)
    M = storage(𝐌)
    if M isa StridedMatrix{Float64} && stride(M, 1) == 1
        return M, stride(M, 2), false
    end
    X = Matrix{Float64}(undef, size(𝐌))
    return X, size(X, 1), true
end
writeback!(𝐌, X, copied) = (copied && copyto!(storage(𝐌), X); 𝐌)

# A spectrum's values as a plain 0-indexed Vector (W[1] is l = 0).
spectrum(V) = collect(Float64, storage(V))

function gpu_mcm!(spin::Cint, 𝐌::FMat, V::SpectralVector{Float64})
    @assert axes(𝐌, 1) == axes(𝐌, 2)
    lmin, lmax = first(axes(𝐌, 1)), last(axes(𝐌, 1))
    M, ld, copied = dense_out(𝐌)  # element (l1,l2) at [l1-lmin+1, l2-lmin+1]
    W = spectrum(V)
    c = ctx()
    st = ccall((:ps_mcm, libps), Cint,
               (Ptr{Cvoid}, Cint, Ptr{Float64}, Int64, Cint, Cint, Cint, Ptr{Float64}, Int64),
               c, spin, W, length(W), lmin, lmax, MODE[], M, ld)
    check(st, c)
    return writeback!(𝐌, M, copied)
end

PowerSpectra.inner_mcm⁰⁰!(𝐌::FMat, V::SpectralVector{Float64}) = gpu_mcm!(PS_SPIN_00, 𝐌, V)
PowerSpectra.inner_mcm⁰²!(𝐌::FMat, V::SpectralVector{Float64}) = gpu_mcm!(PS_SPIN_02, 𝐌, V)
PowerSpectra.inner_mcm⁺⁺!(𝐌::FMat, V::SpectralVector{Float64}) = gpu_mcm!(PS_SPIN_PP, 𝐌, V)
PowerSpectra.inner_mcm⁻⁻!(𝐌::FMat, V::SpectralVector{Float64}) = gpu_mcm!(PS_SPIN_MM, 𝐌, V)

function gpu_cov!(kind::Symbol, 𝐂::FMat, spectra, ratios, windows)
    @assert axes(𝐂, 1) == axes(𝐂, 2)
    lmin, lmax = first(axes(𝐂, 1)), last(axes(𝐂, 1))
    S = [spectrum(x) for x in spectra]
    R = [spectrum(x) for x in ratios]
    W = [spectrum(x) for x in windows]
    nW = minimum(length, W)
    C, ld, copied = dense_out(𝐂)
    c = ctx()
    GC.@preserve S R W begin
        Sp = [pointer(x) for x in S]
        Rp = isempty(R) ? [Ptr{Float64}(C_NULL)] : [pointer(x) for x in R]
        Wp = [pointer(x) for x in W]
        st = ccall((:ps_coupledcov, libps), Cint,
                   (Ptr{Cvoid}, Cint, Ptr{Ptr{Float64}}, Ptr{Ptr{Float64}}, Ptr{Ptr{Float64}}, Int64,
                    Cint, Cint, Cint, Ptr{Float64}, Int64),
                   c, COV[kind], Sp, Rp, Wp, nW, lmin, lmax, MODE[], C, ld)
    end
    check(st, c)
    return writeback!(𝐂, C, copied)
end

const SV = SpectralVector{Float64}

PowerSpectra.loop_covTTTT!(𝐂::FMat, TTip::SV, TTjq::SV, TTiq::SV, TTjp::SV, r_ip::SV, r_jq::SV, r_iq::SV, r_jp::SV,
                           W1, W2, W3, W4, W5, W6, W7, W8) =
    gpu_cov!(:TTTT, 𝐂, (TTip, TTjq, TTiq, TTjp), (r_ip, r_jq, r_iq, r_jp), (W1, W2, W3, W4, W5, W6, W7, W8))
PowerSpectra.loop_covEEEE!(𝐂::FMat, EEip::SV, EEjq::SV, EEiq::SV, EEjp::SV, r_ip::SV, r_jq::SV, r_iq::SV, r_jp::SV,
                           W1, W2, W3, W4, W5, W6, W7, W8) =
    gpu_cov!(:EEEE, 𝐂, (EEip, EEjq, EEiq, EEjp), (r_ip, r_jq, r_iq, r_jp), (W1, W2, W3, W4, W5, W6, W7, W8))
PowerSpectra.loop_covTTTE!(𝐂::FMat, TTip::SV, TTjp::SV, TEiq::SV, TEjq::SV, r_ip::SV, r_jp::SV, W1, W2, W3, W4) =
    gpu_cov!(:TTTE, 𝐂, (TTip, TTjp, TEiq, TEjq), (r_ip, r_jp), (W1, W2, W3, W4))
PowerSpectra.loop_covTETE!(𝐂::FMat, TTip::SV, EEjq::SV, TEiq::SV, TEjp::SV, r_TT_ip::SV, r_PP_jq::SV,
                           W1, W2, W3, W4, W5) =
    gpu_cov!(:TETE, 𝐂, (TTip, EEjq, TEiq, TEjp), (r_TT_ip, r_PP_jq), (W1, W2, W3, W4, W5))
PowerSpectra.loop_covTEEE!(𝐂::FMat, EEjq::SV, EEjp::SV, TEip::SV, TEiq::SV, r_EE_jq::SV, r_EE_jp::SV,
                           W1, W2, W3, W4) =
    gpu_cov!(:TEEE, 𝐂, (EEjq, EEjp, TEip, TEiq), (r_EE_jq, r_EE_jp), (W1, W2, W3, W4))
PowerSpectra.loop_covTEEE_planck!(𝐂::FMat, EEjq::SV, EEjp::SV, TEip::SV, TEiq::SV, r_EE_jq::SV, r_EE_jp::SV,
                                  W1, W2, W3, W4) =
    gpu_cov!(:TEEE_planck, 𝐂, (EEjq, EEjp, TEip, TEiq), (r_EE_jq, r_EE_jp), (W1, W2, W3, W4))
PowerSpectra.loop_covTTEE!(𝐂::FMat, TEip::SV, TEiq::SV, TEjq::SV, TEjp::SV, W1, W2) =
    gpu_cov!(:TTEE, 𝐂, (TEip, TEiq, TEjq, TEjp), (), (W1, W2))

# ---- rows downstream and upstream of the loops ----------------------------------------------

# decouple_covmat (src/covariance.jl:8-14): B1^-1 Y B2^-T by two FP64 LU solves on the GPU
# (the same diagonal signature as the reference's, with T = Float64, so it is the more specific method)
function PowerSpectra.decouple_covmat(Y::SA, B1::SA, B2::SA) where {SA<:FMat}
    M = deepcopy(Y)
    n = size(M, 1)
    Yp, B1p, B2p = (collect(Float64, storage(x)) for x in (Y, B1, B2))  # dense, ld = n
    C, ld, copied = dense_out(M)
    c = ctx()
    st = ccall((:ps_decouple_covmat, libps), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Int64, Int64, Ptr{Float64}, Int64),
               c, Yp, B1p, B2p, n, n, C, ld)
    check(st, c)
    return writeback!(M, C, copied)
end

# quickpolΞ! (src/beam.jl:72-109): quickpolW and the banded Ξ on the GPU; the band is copied
# into the caller's BandedMatrix-backed SpectralArray
function PowerSpectra.quickpolΞ!(𝚵::SpectralArray{Float64,2}, ν₁, ν₂, s₁, s₂,
                                 ω₁::Healpix.Alm{ComplexF64}, ω₂::Healpix.Alm{ComplexF64})
    size(𝚵, 1) != size(𝚵, 2) && throw(ArgumentError("𝚵 is not square."))
    lmax = lastindex(𝚵, 1)
    bl, bu = PowerSpectra.BandedMatrices.bandwidths(parent(𝚵))
    X = Matrix{Float64}(undef, lmax + 1, lmax + 1)
    c = ctx()
    st = ccall((:ps_quickpol_xi_alm, libps), Cint,
               (Ptr{Cvoid}, Cint, Cint, Cint, Cint, Ptr{Float64}, Ptr{Float64}, Cint, Cint, Cint, Cint, Cint, Cint,
                Ptr{Float64}, Int64),
               c, ν₁, ν₂, s₁, s₂, Ptr{Float64}(pointer(ω₁.alm)), Ptr{Float64}(pointer(ω₂.alm)),
               min(ω₁.lmax, ω₂.lmax), min(ω₁.mmax, ω₂.mmax), lmax, bl, bu, MODE[], X, lmax + 1)
    check(st, c)
    for ℓ″ in 2:lmax, ℓ in PowerSpectra.specrowrange(𝚵, ℓ″)
        𝚵[ℓ″, ℓ] = X[ℓ″ + 1, ℓ + 1]
    end
    return 𝚵
end

# window_function_W! (src/workspace.jl:174-213): the alm2cl mean over the weight terms on the
# GPU; the effective-weight coefficients still come from effective_weight_alm! (map2alm)
function PowerSpectra.window_function_W!(workspace::PowerSpectra.CovarianceWorkspace{Float64},
                                         X, Y, i, j, α, p, q, β)
    key = (X, Y, i, j, α, p, q, β)
    haskey(workspace.W_spectra, key) && return workspace.W_spectra[key]
    wterms(Z) = Z == :TT ? (:II,) : (Z == :PP ? (:QQ, :UU) : (Z,))
    A, B = Healpix.Alm{ComplexF64,Vector{ComplexF64}}[], Healpix.Alm{ComplexF64,Vector{ComplexF64}}[]
    for wX in wterms(X), wY in wterms(Y)
        push!(A, PowerSpectra.effective_weight_alm!(workspace, wX, i, j, α))
        push!(B, PowerSpectra.effective_weight_alm!(workspace, wY, p, q, β))
    end
    lmax = workspace.lmax
    result = zeros(Float64, lmax + 1)
    c = ctx()
    GC.@preserve A B begin
        pa = [Ptr{Float64}(pointer(a.alm)) for a in A]
        pb = [Ptr{Float64}(pointer(b.alm)) for b in B]
        st = ccall((:ps_window_W, libps), Cint,
                   (Ptr{Cvoid}, Ptr{Ptr{Float64}}, Ptr{Ptr{Float64}}, Cint, Cint, Cint, Cint, Ptr{Float64}),
                   c, pa, pb, length(A), A[1].lmax, A[1].mmax, lmax, result)
        check(st, c)
    end
    W = SpectralVector(result)
    workspace.W_spectra[key] = W
    return W
end

function __init__()
    atexit() do
        for (_, h) in CTXS
            ccall((:ps_destroy, libps), Cvoid, (Ptr{Cvoid},), h)
        end
    end
end

end # module
