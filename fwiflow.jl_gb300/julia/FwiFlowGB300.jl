# Julia binding of the GB300 elastic FWI operator (libfwiflow_gb300.so).
#
# Gives FwiFlow.jl's operator surface without TensorFlow:
#   fwi_op / fwi_obs_op                      src/Core.jl:20-53 (shot_ids 0-based, λ, μ in MPa)
#   compute_observation / compute_misfit     src/FWI.jl:109-189 (shot_ids 1-based, velocities)
#   velocity_to_moduli                       src/Utils.jl:221-227
# and a ChainRulesCore rrule for fwi_op whose pullback multiplies the
# gradients by the incoming cotangent (FwiOpGrad, FwiOp.cpp:207-222, passes
# them through unscaled).
#
# Layout: the C ABI takes row-major [nz][nx] doubles with (z, x) indexing, as
# the TF op receives them. A Julia Matrix (nz, nx) is column-major, so every
# model array crosses the boundary as permutedims(A) (an (nx, nz) array whose
# memory is the row-major (nz, nx) array), and gradients come back the same
# way. stf (nShots, nSteps) likewise.
#
# Julia is not available where this package is built and tested; the file is
# written against the C ABI declared in include/fwiflow_gb300.h.
module FwiFlowGB300

using ChainRulesCore

export fwi_op, fwi_op_grad, fwi_obs_op, compute_observation, compute_misfit, velocity_to_moduli,
       FwiContext, close_context

const LIB = Ref{String}(joinpath(@__DIR__, "..", "_build", "libfwiflow_gb300.so"))

"Path of the shared library (override before the first call if it lives elsewhere)."
set_library!(path::AbstractString) = (LIB[] = String(path))

mutable struct FwiContext
    handle::Ptr{Cvoid}
    para_fname::String
    gpu_id::Int
    nz::Int
    nx::Int
    nSteps::Int
    nrec_max::Int
end

function _check(st::Cint, ctx::Union{Nothing,FwiContext}=nothing)
    st == 0 && return nothing
    msg = ctx === nothing ?
        unsafe_string(ccall((:fwigb_last_global_error, LIB[]), Cstring, ())) :
        unsafe_string(ccall((:fwigb_last_error, LIB[]), Cstring, (Ptr{Cvoid},), ctx.handle))
    error("fwiflow_gb300 status $st: $msg")
end

function FwiContext(para_fname::AbstractString, gpu_id::Integer=0)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    _check(ccall((:fwigb_create, LIB[]), Cint, (Cstring, Cint, Ptr{Ptr{Cvoid}}), para_fname, gpu_id, h))
    nz, nx, nt, nsh, nrm = Ref{Cint}(0), Ref{Cint}(0), Ref{Cint}(0), Ref{Cint}(0), Ref{Cint}(0)
    ctx = FwiContext(h[], String(para_fname), Int(gpu_id), 0, 0, 0, 0)
    _check(ccall((:fwigb_geometry, LIB[]), Cint,
                 (Ptr{Cvoid}, Ref{Cint}, Ref{Cint}, Ref{Cint}, Ref{Cint}, Ref{Cint}), h[], nz, nx, nt, nsh, nrm), ctx)
    ctx.nz, ctx.nx, ctx.nSteps, ctx.nrec_max = nz[], nx[], nt[], nrm[]
    finalizer(close_context, ctx)
    ctx
end

function close_context(ctx::FwiContext)
    if ctx.handle != C_NULL
        ccall((:fwigb_destroy, LIB[]), Cvoid, (Ptr{Cvoid},), ctx.handle)
        ctx.handle = C_NULL
    end
    nothing
end

# One context per (parameter file, GPU), kept across calls like the library's
# own cache behind fwigb_cufd.
const _CONTEXTS = Dict{Tuple{String,Int},FwiContext}()
function _ctx(para_fname::AbstractString, gpu_id::Integer)
    key = (abspath(para_fname), Int(gpu_id))
    get!(() -> FwiContext(para_fname, gpu_id), _CONTEXTS, key)
end

_rowmajor(A::AbstractMatrix) = Matrix{Float64}(permutedims(A))        # (nz,nx) -> memory [nz][nx]
_colmajor(B::Matrix{Float64}) = Matrix{Float64}(permutedims(B))       # back to (nz,nx)

function _shape_check(ctx::FwiContext, A)
    size(A) == (ctx.nz, ctx.nx) || error("model arrays must be ($(ctx.nz), $(ctx.nx)), got $(size(A))")
end

"""
    fwi_op(λ, μ, ρ, stf, gpu_id, shot_ids, para_fname) -> misfit::Float64

Misfit of the elastic FWI operator (cufd calc_id 0). λ, μ in MPa, ρ in kg/m³,
all (nz, nx) with the CPML padding; stf (nShots, nSteps); shot_ids 0-based.
"""
function fwi_op(λ::AbstractMatrix, μ::AbstractMatrix, ρ::AbstractMatrix, stf::AbstractMatrix,
                gpu_id::Integer, shot_ids::AbstractVector{<:Integer}, para_fname::AbstractString)
    ctx = _ctx(para_fname, gpu_id)
    foreach(A -> _shape_check(ctx, A), (λ, μ, ρ))
    misfit = Ref{Float64}(0.0)
    ids = Int32.(shot_ids)
    _check(ccall((:fwigb_misfit, LIB[]), Cint,
                 (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Cint, Ptr{Int32}, Cint,
                  Ref{Float64}),
                 ctx.handle, _rowmajor(λ), _rowmajor(μ), _rowmajor(ρ), _rowmajor(stf), size(stf, 1), ids,
                 length(ids), misfit), ctx)
    misfit[]
end

"""
    fwi_op_grad(λ, μ, ρ, stf, gpu_id, shot_ids, para_fname) -> (misfit, gλ, gμ, gρ, gstf)

Misfit and its gradients from one forward and one adjoint sweep (cufd
calc_id 1). gstf has the shape of stf with the first length(shot_ids) rows
filled in shot order (libCUFD.cu:452-456).
"""
function fwi_op_grad(λ::AbstractMatrix, μ::AbstractMatrix, ρ::AbstractMatrix, stf::AbstractMatrix,
                     gpu_id::Integer, shot_ids::AbstractVector{<:Integer}, para_fname::AbstractString)
    ctx = _ctx(para_fname, gpu_id)
    foreach(A -> _shape_check(ctx, A), (λ, μ, ρ))
    ids = Int32.(shot_ids)
    misfit = Ref{Float64}(0.0)
    gλ, gμ, gρ = (zeros(ctx.nx, ctx.nz) for _ in 1:3)          # row-major [nz][nx] memory
    gs = zeros(size(stf, 2), length(ids))                        # row-major [n_shots][nSteps]
    _check(ccall((:fwigb_misfit_grad, LIB[]), Cint,
                 (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Cint, Ptr{Int32}, Cint,
                  Ref{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                 ctx.handle, _rowmajor(λ), _rowmajor(μ), _rowmajor(ρ), _rowmajor(stf), size(stf, 1), ids,
                 length(ids), misfit, gλ, gμ, gρ, gs), ctx)
    gstf = zeros(size(stf))
    gstf[1:length(ids), :] = permutedims(gs)
    misfit[], _colmajor(gλ), _colmajor(gμ), _colmajor(gρ), gstf
end

"""
    fwi_obs_op(λ, μ, ρ, stf, gpu_id, shot_ids, para_fname) -> 0.0

Forward modelling (cufd calc_id 2): writes data_dir_name/Shot<id>.bin for
every shot, [nrec][nSteps] Float32 (libCUFD.cu:514-521), and returns 0.0.
"""
function fwi_obs_op(λ::AbstractMatrix, μ::AbstractMatrix, ρ::AbstractMatrix, stf::AbstractMatrix,
                    gpu_id::Integer, shot_ids::AbstractVector{<:Integer}, para_fname::AbstractString)
    ctx = _ctx(para_fname, gpu_id)
    foreach(A -> _shape_check(ctx, A), (λ, μ, ρ))
    ids = Int32.(shot_ids)
    _check(ccall((:fwigb_obs, LIB[]), Cint,
                 (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Cint, Ptr{Int32}, Cint,
                  Ptr{Float32}, Cint),
                 ctx.handle, _rowmajor(λ), _rowmajor(μ), _rowmajor(ρ), _rowmajor(stf), size(stf, 1), ids,
                 length(ids), C_NULL, 1), ctx)
    0.0
end

function ChainRulesCore.rrule(::typeof(fwi_op), λ, μ, ρ, stf, gpu_id, shot_ids, para_fname)
    J, gλ, gμ, gρ, gstf = fwi_op_grad(λ, μ, ρ, stf, gpu_id, shot_ids, para_fname)
    function fwi_op_pullback(ȳ)
        s = unthunk(ȳ)
        return (NoTangent(), s .* gλ, s .* gμ, s .* gρ, s .* gstf, NoTangent(), NoTangent(), NoTangent())
    end
    return J, fwi_op_pullback
end

"λ, μ in MPa from cp, cs [m/s] and ρ (src/Utils.jl:221-227)."
function velocity_to_moduli(cp, cs, ρ)
    λ = (cp .^ 2 .- 2 .* cs .^ 2) .* ρ ./ 1e6
    μ = cs .^ 2 .* ρ ./ 1e6
    λ, μ
end

"""
    compute_observation(para_fname, cp, cs, ρ, stf, shot_ids; gpu_id=0) -> data (n_shots, nSteps, nrec)

Velocities on the padded grid; shot_ids 1-based as in src/FWI.jl:109-136.
The gathers are returned (and written to Data/Shot<id>.bin) with the
reference's (shot, time, receiver) layout.
"""
function compute_observation(para_fname::AbstractString, cp, cs, ρ, stf::AbstractMatrix,
                             shot_ids::AbstractVector{<:Integer}; gpu_id::Integer=0)
    ctx = _ctx(para_fname, gpu_id)
    λ, μ = velocity_to_moduli(cp, cs, ρ)
    ids = Int32.(shot_ids .- 1)
    buf = zeros(Float32, ctx.nSteps, ctx.nrec_max, length(ids))   # [shot][nrec][nSteps] row-major
    _check(ccall((:fwigb_obs, LIB[]), Cint,
                 (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Cint, Ptr{Int32}, Cint,
                  Ptr{Float32}, Cint),
                 ctx.handle, _rowmajor(λ), _rowmajor(μ), _rowmajor(ρ), _rowmajor(stf), size(stf, 1), ids,
                 length(ids), buf, 1), ctx)
    data = zeros(length(ids), ctx.nSteps, ctx.nrec_max)
    for i in eachindex(ids)
        data[i, :, :] = buf[:, :, i]
    end
    data
end

"""
    compute_misfit(para_fname, cp, cs, ρ, stf, shot_ids; gpu_id=0, mask=nothing, cp_ref, cs_ref, ρ_ref)

Misfit for velocities on the padded grid (src/FWI.jl:138-189). With `mask`
(1 inside the inverted region, 0 outside) the model outside is taken from
the reference model, as the reference's masking does.
"""
function compute_misfit(para_fname::AbstractString, cp, cs, ρ, stf::AbstractMatrix,
                        shot_ids::AbstractVector{<:Integer}; gpu_id::Integer=0, mask=nothing,
                        cp_ref=nothing, cs_ref=nothing, ρ_ref=nothing)
    if mask !== nothing
        cp = cp .* mask .+ cp_ref .* (1 .- mask)
        cs = cs .* mask .+ cs_ref .* (1 .- mask)
        ρ = ρ .* mask .+ ρ_ref .* (1 .- mask)
    end
    λ, μ = velocity_to_moduli(cp, cs, ρ)
    fwi_op(λ, μ, ρ, stf, gpu_id, shot_ids .- 1, para_fname)
end

end # module
