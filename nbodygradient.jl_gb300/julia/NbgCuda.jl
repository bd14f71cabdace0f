# NbgCuda.jl -- routes NbodyGradient.jl's transit-timing integration through
# libnbg_cuda (the GB300 implementation of this package).
#
# Loading this file after `using NbodyGradient` adds methods, more specific
# than the reference's, for Float64 states and the ahl21! scheme:
#   intr(s, tt::TransitTiming; grad)        (src/transits/Transits.jl:173-180)
#   intr(s, ttbv::TransitParameters; grad)  (same, TransitParameters output)
#   intr(s, tt, d::Derivatives; grad)       (src/transits/Transits.jl:140, both outputs)
#   intr(s, time::Float64; grad)            (src/integrator/Integrator.jl:159)
#   intr(s, N::Int64; grad)                 (src/integrator/Integrator.jl:210)
#   intr(s, o::CartesianOutput)             (src/outputs/Outputs.jl:26)
# (intr(s; grad) reaches the GPU through intr(s, time).)  Everything else
# stays on the reference's own code path.  The library path comes from
# ENV["NBG_CUDA_LIB"].
#
# Not exercised in this repository's test suite (Julia is not installed on
# the build and GPU hosts); tests drive the same C ABI from Python.
module NbgCuda

using NbodyGradient
import NbodyGradient: Integrator, State, TransitTiming, TransitParameters, CartesianOutput, ahl21!, check_step

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

const NBG_ENONFINITE = -5

# A non-zero return code becomes an error, except NBG_ENONFINITE: the
# reference lets non-finite values propagate into the State silently, so the
# shim keeps the call's (written) outputs and only warns.
function check_rc(rc)
    rc == 0 && return
    rc == NBG_ENONFINITE && (@warn "libnbg_cuda: " * last_error(); return)
    error("libnbg_cuda: ", last_error())
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
    check_rc(rc)
    # the step scratch for later three-argument calls (Transits.jl:176-178); this
    # path keeps its scratch on the device, so a fresh one is handed back
    return_arrays && return NbodyGradient.Derivatives(Float64, s.n)
    return nothing
end

function (intr::Integrator{Float64,typeof(ahl21!)})(s::State{Float64}, ttbv::TransitParameters{Float64};
                                                    grad::Bool=true, return_arrays::Bool=false)
    GC.@preserve s ttbv begin
        rc = ccall((:nbg_integrate_transit_parameters, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cint, Cdouble, Cdouble, Cint,
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Bool}, Ptr{Float64}, Int64,
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Int64}),
                   context(), s.n, ttbv.ti - 1, intr.h, intr.tmax, grad ? 1 : 0,
                   s.t, s.x, s.v, s.m, s.xerror, s.verror,
                   s.jac_step, s.jac_error, s.dqdt, s.pair, s.jac_init, ttbv.ntt,
                   ttbv.ttbv, ttbv.dtbvdq0, ttbv.dtbvdelements, ttbv.count)
    end
    check_rc(rc)
    return_arrays && return NbodyGradient.Derivatives(Float64, s.n)
    return nothing
end

# The three-argument forms with preallocated Derivatives (Transits.jl:140,
# e.g. after dState(ic)) take the same GPU path; the scratch lives on the
# device, so d is not used.
function (intr::Integrator{Float64,typeof(ahl21!)})(s::State{Float64}, tt::TransitTiming{Float64},
                                                    d::NbodyGradient.Derivatives{Float64}; grad::Bool=true)
    return intr(s, tt; grad=grad)
end

function (intr::Integrator{Float64,typeof(ahl21!)})(s::State{Float64}, ttbv::TransitParameters{Float64},
                                                    d::NbodyGradient.Derivatives{Float64}; grad::Bool=true)
    return intr(s, ttbv; grad=grad)
end

# ccall's argument types must be a literal tuple, so the State pointers
# (t, x, v, m, xerror, verror, jac_step, jac_error, dqdt, pair) are spelled out.
function (intr::Integrator{Float64,typeof(ahl21!)})(s::State{Float64}, time::Float64; grad::Bool=true)
    GC.@preserve s begin
        rc = ccall((:nbg_integrate, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cdouble, Cdouble, Cint,
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Bool}),
                   context(), s.n, intr.h, time, grad ? 1 : 0,
                   s.t, s.x, s.v, s.m, s.xerror, s.verror, s.jac_step, s.jac_error, s.dqdt, s.pair)
    end
    check_rc(rc)
    return
end

function (intr::Integrator{Float64,typeof(ahl21!)})(s::State{Float64}, N::Int64; grad::Bool=true)
    GC.@preserve s begin
        rc = ccall((:nbg_integrate_steps, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cdouble, Int64, Cint,
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Bool}),
                   context(), s.n, intr.h, N, grad ? 1 : 0,
                   s.t, s.x, s.v, s.m, s.xerror, s.verror, s.jac_step, s.jac_error, s.dqdt, s.pair)
    end
    check_rc(rc)
    intr.h < 0 && (intr.h = -intr.h)  # as the reference leaves it (Integrator.jl:228-229)
    return
end

function (intr::Integrator{Float64,typeof(ahl21!)})(s::State{Float64}, o::CartesianOutput{Float64})
    n, M, nstep = s.n, 7 * s.n, o.nstep
    ts = Vector{Float64}(undef, nstep)
    xs = Array{Float64}(undef, 3, n, nstep)
    vs = Array{Float64}(undef, 3, n, nstep)
    js = Array{Float64}(undef, M, M, nstep)
    GC.@preserve s begin
        rc = ccall((:nbg_integrate_cartesian, LIB), Cint,
                   (Ptr{Cvoid}, Cint, Cdouble, Cdouble, Int64,
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64},
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Bool},
                    Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                   context(), n, intr.h, intr.tmax, nstep,
                   s.t, s.x, s.v, s.m, s.xerror, s.verror, s.jac_step, s.jac_error, s.dqdt, s.pair,
                   ts, xs, vs, js)
    end
    check_rc(rc)
    for i in 1:nstep  # o.states[i] = the state before step i (Outputs.jl:38-40)
        si = deepcopy(s)
        si.t[1] = ts[i]; si.x .= xs[:, :, i]; si.v .= vs[:, :, i]; si.jac_step .= js[:, :, i]
        o.states[i] = si
    end
    return
end

end # module
