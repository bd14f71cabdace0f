# NbgCuda.jl -- routes NbodyGradient.jl's transit-timing integration through
# libnbg_cuda (the GB300 implementation of this package).
#
# Loading this file after `using NbodyGradient` adds a method, more specific
# than (intr::Integrator)(s::State, tt::TransitOutput; grad, return_arrays)
# (src/transits/Transits.jl:173-180), for Float64 states, TransitTiming
# outputs and the ahl21! scheme.  Everything else stays on the reference's
# own code path.  The library path comes from ENV["NBG_CUDA_LIB"].
#
# Not exercised in this repository's test suite (Julia is not installed on
# the build and GPU hosts); tests drive the same C ABI from Python.
module NbgCuda

using NbodyGradient
import NbodyGradient: Integrator, State, TransitTiming, ahl21!

const LIB = get(ENV, "NBG_CUDA_LIB", "libnbg_cuda.so")
const CTX = Ref{Ptr{Cvoid}}(C_NULL)

function context()
    if CTX[] == C_NULL
        h = Ref{Ptr{Cvoid}}(C_NULL)
        rc = ccall((:nbg_create, LIB), Cint, (Cint, Ref{Ptr{Cvoid}}), 0, h)
        rc == 0 || error("nbg_create failed: ", last_error())
        CTX[] = h[]
    end
    return CTX[]
end

function last_error()
    buf = Vector{UInt8}(undef, 512)
    ccall((:nbg_last_error, LIB), Cint, (Ptr{UInt8}, Csize_t), buf, length(buf))
    return unsafe_string(pointer(buf))
end

function (intr::Integrator{Float64,typeof(ahl21!)})(s::State{Float64}, tt::TransitTiming{Float64};
                                                    grad::Bool=true, return_arrays::Bool=false)
    t = s.t  # Vector{Float64} of length 1, updated in place
    GC.@preserve s tt begin
        rc = ccall((:nbg_integrate_transits, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cint, Cdouble, Cdouble, Cint,
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Bool}, Ptr{Float64}, Int64,
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int64}),
                   context(), s.n, tt.ti - 1, intr.h, intr.tmax, grad ? 1 : 0,
                   t, s.x, s.v, s.m, s.xerror, s.verror,
                   s.jac_step, s.jac_error, s.dqdt, s.pair, s.jac_init, tt.ntt,
                   tt.tt, tt.dtdq0, tt.dtdelements, tt.count)
    end
    rc == 0 || error("libnbg_cuda: ", last_error())
    return_arrays && return nothing  # no Derivatives scratch exists on this path
    return nothing
end

end # module
