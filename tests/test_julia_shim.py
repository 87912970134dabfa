"""Static checks of the Julia ccall shim (Julia is not installed, so the shim is
read as text).

The shim must override the reference's loops for the matrices `mcm` and
`coupledcov` really pass: spectralzeros(lmin:lmax, lmin:lmax)
(src/spectralarray.jl:74, src/modecoupling.jl:199, src/covariance.jl:38) has
an OffsetArray parent, so a method pinned to a Matrix parent would never be
selected and the reference's CPU loops would run silently.  Its default
arithmetic must be FP64, like the reference's loops.
"""
import os
import re

from conftest import PKG

SHIM = os.path.join(PKG, "julia", "PowerSpectraGPU.jl")


def _src():
    return open(SHIM, encoding="utf-8").read()


def _code(src):
    return "\n".join(line.split("#", 1)[0] for line in src.splitlines())


def test_no_override_pins_the_matrix_parent_type():
    code = _code(_src())
    assert not re.search(r"SpectralArray\{\s*Float64\s*,\s*2\s*,", code), \
        "an override pins the storage type of SpectralArray"
    assert re.search(r"const FMat = SpectralArray\{Float64,\s*2\}\s*$", code, flags=re.M)


def test_every_loop_is_overridden_on_fmat():
    code = _code(_src())
    for name in ("inner_mcm⁰⁰!", "inner_mcm⁰²!", "inner_mcm⁺⁺!", "inner_mcm⁻⁻!", "loop_covTTTT!", "loop_covEEEE!",
                 "loop_covTTTE!", "loop_covTETE!", "loop_covTEEE!", "loop_covTEEE_planck!", "loop_covTTEE!"):
        m = re.search(r"PowerSpectra\.%s\((\S+?)::(\w+)" % re.escape(name), code)
        assert m, name
        assert m.group(2) == "FMat", (name, m.group(2))
    # decouple_covmat keeps the reference's diagonal signature with T = Float64
    assert re.search(r"decouple_covmat\(Y::SA, B1::SA, B2::SA\) where \{SA<:FMat\}", code)


def test_outputs_are_written_through_the_innermost_storage():
    code = _code(_src())
    # the pointer handed to ccall is the dense storage with its own leading dimension
    assert "stride(M, 1) == 1" in code and "stride(M, 2)" in code
    assert code.count("writeback!(") >= 3
    assert "parent(𝐌)" not in code and "parent(𝐂)" not in code


def test_default_mode_is_fp64():
    code = _code(_src())
    m = re.search(r"const MODE = Ref\((\w+)\)", code)
    assert m and m.group(1) == "PS_MODE_PLAIN_FP64"
