# QuantumBilliardsGPU.jl — Julia binding of libqbgpu (ccall shim).
#
# Adds GPU methods to QuantumBilliards.jl's own functions for a wrapper solver
# type, so existing driver code (k_sweep, compute_spectrum_beyn, EBIM) keeps
# its signatures:
#   construct_matrices!           (dlp_kress.jl:1627-1679, cfie_kress.jl:893-929)
#   construct_boundary_matrices!  (chebyshev_euclidian_helmholtz_{dlp,cfie}_kress.jl)
#   construct_B_matrix            (beyn.jl:257-322)
# Julia is not installed where this project is built and tested; this file is
# the binding a maintainer adds, written against include/qbgpu.h.
module QuantumBilliardsGPU

using LinearAlgebra
import QuantumBilliards
const QB = QuantumBilliards

const libqbgpu = get(ENV, "QBGPU_LIB", joinpath(@__DIR__, "..", "qbgpu", "libqbgpu.so"))

const QBG_FORM_DLP = Int32(0)
const QBG_FORM_CFIE = Int32(1)
const QBG_PREC_FP64 = Int32(0)
const QBG_PREC_MIXED = Int32(1)

struct QbgGeomDesc
    form::Int32
    ncomp::Int32
    comp_offsets::Ptr{Int64}
    x::Ptr{Float64}; y::Ptr{Float64}
    dx::Ptr{Float64}; dy::Ptr{Float64}
    ddx::Ptr{Float64}; ddy::Ptr{Float64}
    ts::Ptr{Float64}; ws::Ptr{Float64}
    m::Int64; norb::Int32
    fund::Ptr{Int64}; orbit::Ptr{Int64}; orbit_scale::Ptr{Float64}
    quad::Int32                      # 0 = Kress, 1 = Alpert (cache built by the caller)
    alpert_a::Int32; alpert_j::Int32; alpert_ninterp::Int32
    alpert_w::Ptr{Float64}; alpert_off::Ptr{Int64}; alpert_wt::Ptr{Float64}; alpert_nodes::Ptr{Float64}
end

struct QbgChebParams
    n_panels_h::Int32
    M_h::Int32
    n_panels_j::Int32
    M_j::Int32
end

struct QbgBeynOpts
    flags::Int32
    max_refine::Int32
    refine_tol::Float64
    nb::Int32
    eval_mode::Int32        # 0 = Chebyshev panels (use_chebyshev=true), 1 = direct
    cheb::QbgChebParams     # zeros = the reference defaults 15000, 5, 3000, 5
    fp32_sweeps::Int32      # complex64 forms: plain FP32 residual corrections (0 = default)
    solve_block::Int32      # complex64 forms: triangular-solve block rows (0 = default)
    node_chunk::Int32       # 0: all node operators resident; c > 0: stream the nodes c at a time
    resid_engine::Int32     # 0: tensor-core residual (digit products), 1: compensated FP32
end

function qbg_check(st::Int32)
    st == 0 && return nothing
    buf = Vector{UInt8}(undef, 2048)
    ccall((:qbg_last_error, libqbgpu), Csize_t, (Ptr{UInt8}, Csize_t), buf, length(buf))
    error("qbgpu: status $(st): " * unsafe_string(pointer(buf)))
end

"Wrapper solver: routes the hot path of `S` to the GPU."
struct GPUSolver{S}
    inner::S
    prec::Int32
end
GPUSolver(s; mixed::Bool=false) = GPUSolver(s, mixed ? QBG_PREC_MIXED : QBG_PREC_FP64)

mutable struct GPUWorkspace
    h::Ptr{Cvoid}
    dim::Int
    keep::Vector{Any}   # host arrays referenced during creation
    function GPUWorkspace(h, dim, keep)
        ws = new(h, dim, keep)
        finalizer(w -> ccall((:qbg_geom_destroy, libqbgpu), Int32, (Ptr{Cvoid},), w.h), ws)
        ws
    end
end

_form(::Union{QB.DLP_kress,QB.DLP_kress_global_corners}) = QBG_FORM_DLP
_form(::Union{QB.CFIE_kress,QB.CFIE_kress_corners,QB.CFIE_kress_global_corners}) = QBG_FORM_CFIE

"Upload a discretisation (BoundaryPointsCFIE or a vector of them)."
function gpu_workspace(solver::GPUSolver, pts)
    comps = pts isa AbstractVector ? pts : [pts]
    offs = Int64[0]
    for p in comps
        push!(offs, offs[end] + length(p.xy))
    end
    cat(f) = reduce(vcat, [f(p) for p in comps])
    x = cat(p -> getindex.(p.xy, 1)); y = cat(p -> getindex.(p.xy, 2))
    dx = cat(p -> getindex.(p.tangent, 1)); dy = cat(p -> getindex.(p.tangent, 2))
    ddx = cat(p -> getindex.(p.tangent_2, 1)); ddy = cat(p -> getindex.(p.tangent_2, 2))
    ts = cat(p -> p.ts); wsv = cat(p -> p.ws)
    keep = Any[offs, x, y, dx, dy, ddx, ddy, ts, wsv]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve keep begin
        d = QbgGeomDesc(_form(solver.inner), Int32(length(comps)), pointer(offs), pointer(x), pointer(y),
                        pointer(dx), pointer(dy), pointer(ddx), pointer(ddy), pointer(ts), pointer(wsv),
                        0, 0, C_NULL, C_NULL, C_NULL,
                        0, 0, 0, 0, C_NULL, C_NULL, C_NULL, C_NULL)  # Kress; an Alpert solver fills the cache fields
        qbg_check(ccall((:qbg_geom_create, libqbgpu), Int32, (Ref{QbgGeomDesc}, Ref{Ptr{Cvoid}}), d, h))
    end
    dim = Ref{Int64}(0)
    qbg_check(ccall((:qbg_geom_dim, libqbgpu), Int32, (Ptr{Cvoid}, Ref{Int64}), h[], dim))
    return GPUWorkspace(h[], Int(dim[]), keep)
end

# construct_boundary_matrices!(Tbufs, solver, pts, zj; ...) — complex k, multi-k
function QB.construct_boundary_matrices!(Tbufs::Vector{Matrix{ComplexF64}}, solver::GPUSolver, pts,
                                         zj::AbstractVector{ComplexF64}; kwargs...)
    ws = gpu_workspace(solver, pts)
    ptrs = [pointer(T) for T in Tbufs]
    GC.@preserve Tbufs zj qbg_check(ccall((:qbg_assemble, libqbgpu), Int32,
        (Ptr{Cvoid}, Ptr{ComplexF64}, Int64, Int32, Int32, Int32, Ptr{Ptr{ComplexF64}}),
        ws.h, collect(zj), length(zj), 0, QBG_PREC_FP64, 0, ptrs))
    return nothing
end

# construct_matrices!(solver, A, dA, ddA, pts, ws, k) — real k with derivatives (EBIM, Newton)
function QB.construct_matrices!(solver::GPUSolver, A::Matrix{ComplexF64}, dA::Matrix{ComplexF64},
                                ddA::Matrix{ComplexF64}, pts, ws::GPUWorkspace, k::Real; kwargs...)
    kk = ComplexF64[k]
    ptrs = [pointer(A), pointer(dA), pointer(ddA)]
    GC.@preserve A dA ddA kk qbg_check(ccall((:qbg_assemble, libqbgpu), Int32,
        (Ptr{Cvoid}, Ptr{ComplexF64}, Int64, Int32, Int32, Int32, Ptr{Ptr{ComplexF64}}),
        ws.h, kk, 1, 1, QBG_PREC_FP64, 0, ptrs))
    return A, dA, ddA
end

# construct_B_matrix(solver, pts, N, k0, R; nq, r, svd_tol, rng) — beyn.jl:257-322,
# with the N^2 / N^3 work on the GPU and the small SVD / B on the host.
function QB.construct_B_matrix(solver::GPUSolver, pts, N::Int, k0::Complex{Float64}, R::Float64;
                               nq::Int=64, r::Int=48, svd_tol=1e-14, rng=QB.MersenneTwister(0), kwargs...)
    ws = gpu_workspace(solver, pts)
    @assert ws.dim == N
    h = Ref{Ptr{Cvoid}}(C_NULL)
    opts = QbgBeynOpts(0, 10, 1e-6, 0, 0, QbgChebParams(0, 0, 0, 0), 0, 0, 0, 0)
    qbg_check(ccall((:qbg_beyn_create, libqbgpu), Int32,
        (Ptr{Cvoid}, Float64, Float64, Float64, Int32, Int32, Ref{QbgBeynOpts}, Ref{Ptr{Cvoid}}),
        ws.h, real(k0), imag(k0), R, nq, solver.prec, opts, h))
    moments(V) = begin
        A0 = similar(V); A1 = similar(V)
        GC.@preserve V A0 A1 qbg_check(ccall((:qbg_beyn_moments, libqbgpu), Int32,
            (Ptr{Cvoid}, Ptr{ComplexF64}, Int64, Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{Cvoid}),
            h[], V, size(V, 2), A0, A1, C_NULL))
        A0, A1
    end
    try
        V = randn(rng, ComplexF64, N, r)
        A0, A1 = moments(V)
        U, Σ, W = svd!(A0; full=false)
        rk = count(>=(svd_tol), Σ)
        rk == 0 && return Matrix{ComplexF64}(undef, N, 0), Matrix{ComplexF64}(undef, N, 0)
        if rk == r && 2r < N
            V = randn(rng, ComplexF64, N, 2r)
            A0, A1 = moments(V)
            U, Σ, W = svd!(A0; full=false)
            rk = count(>=(svd_tol), Σ)
        end
        Uk = U[:, 1:rk]; Wk = W[:, 1:rk]
        tmp = (A1 * Wk) ./ transpose(Σ[1:rk])
        return Uk' * tmp, Uk
    finally
        ccall((:qbg_beyn_destroy, libqbgpu), Int32, (Ptr{Cvoid},), h[])
    end
end

# EBIM eigen step on given matrices — solve_krylov! (ebim.jl:464-537) and
# solve_full! (ebim.jl:336-375); the reference dispatches them on EBIMSolver,
# so a caller holding A, dA, ddA calls these directly (or adds the two one-line
# methods for its own solver wrapper). Returns (k_corrected, tensions).
const QBG_EBIM_FULL = Int32(8)
function gpu_ebim(A::Matrix{ComplexF64}, dA::Matrix{ComplexF64}, ddA::Matrix{ComplexF64}, k::Real, dk::Real;
                  nev::Int=5, full::Bool=false, return_imag_part::Bool=false)
    n = size(A, 1)
    cap = max(nev, 8)
    while true
        out = zeros(Float64, 2cap); tens = zeros(Float64, cap); cnt = Ref{Int32}(0)
        GC.@preserve A dA ddA out tens qbg_check(ccall((:qbg_ebim_eig, libqbgpu), Int32,
            (Int64, Ptr{ComplexF64}, Ptr{ComplexF64}, Ptr{ComplexF64}, Float64, Float64, Int32, Int32, Int32,
             Ptr{Float64}, Ptr{Float64}, Ref{Int32}, Ptr{Int32}),
            n, A, dA, ddA, k, dk, nev, full ? QBG_EBIM_FULL : Int32(0), cap, out, tens, cnt, C_NULL))
        m = Int(cnt[])
        if m <= cap
            kc = [complex(out[2i - 1], out[2i]) for i in 1:m]
            return (return_imag_part ? kc : real.(kc)), tens[1:m]
        end
        cap = m
    end
end
QB.solve_krylov!(solver::GPUSolver, A, dA, ddA, pts, k, dk; nev::Int=5, return_imag_part::Bool=false, kwargs...) =
    gpu_ebim(A, dA, ddA, k, dk; nev=nev, return_imag_part=return_imag_part)
QB.solve_full!(solver::GPUSolver, A, dA, ddA, pts, k, dk; return_imag_part::Bool=false, kwargs...) =
    gpu_ebim(A, dA, ddA, k, dk; full=true, return_imag_part=return_imag_part)

# solve!(solver, A, dA, ddA, pts, k, dk; use_krylov, nev) (ebim.jl:931-939): one
# EBIM window, assembly and eigen step on the GPU.
function QB.solve!(solver::GPUSolver, A::Matrix{ComplexF64}, dA::Matrix{ComplexF64}, ddA::Matrix{ComplexF64},
                   pts, k::Real, dk::Real; use_krylov::Bool=true, nev::Int=5, return_imag_part::Bool=false,
                   kwargs...)
    ws = gpu_workspace(solver, pts)
    QB.construct_matrices!(solver, A, dA, ddA, pts, ws, k)
    return gpu_ebim(A, dA, ddA, k, dk; nev=nev, full=!use_krylov, return_imag_part=return_imag_part)
end

# newton_refine_svd! (sweepmethods.jl:307-368) on the workspace's discretisation:
# the reference's closure-based version assembles on the host; this one keeps
# A, A', A'' and A^H A on the device. Returns (k, tension).
function gpu_newton_refine(ws::GPUWorkspace, k0::Real; a::Real=0.0, b::Real=Inf, maxiter::Int=8, tol::Real=1e-12)
    kout = Ref{Float64}(0); tout = Ref{Float64}(0)
    qbg_check(ccall((:qbg_newton_refine, libqbgpu), Int32,
        (Ptr{Cvoid}, Float64, Float64, Float64, Int32, Float64, Ref{Float64}, Ref{Float64}, Ptr{Int32}),
        ws.h, k0, a, b, maxiter, tol, kout, tout, C_NULL))
    return kout[], tout[]
end

# adjoint_fredholm_matrix!(A, D, solver, pts, ws, k) (dlp_kress.jl:1451-1500) and
# solve_vect(solver, basis, pts, ws, k) (dlp_kress.jl:1914-1949) for the DLP
# forms: the adjoint matrix and the smallest null vector on the device.
function QB.adjoint_fredholm_matrix!(A::Matrix{ComplexF64}, D::AbstractMatrix{ComplexF64}, solver::GPUSolver,
                                     pts, ws::GPUWorkspace, k::Real; kwargs...)
    ds = collect(Float64, pts.ds)
    GC.@preserve A ds qbg_check(ccall((:qbg_adjoint_fredholm, libqbgpu), Int32,
        (Ptr{Cvoid}, Float64, Ptr{Float64}, Ptr{ComplexF64}, Int32), ws.h, k, ds, A, Int32(0)))
    return A
end
function QB.solve_vect(solver::GPUSolver, basis::QB.AbsBasis, pts, ws::GPUWorkspace, k::Real; kwargs...)
    ds = collect(Float64, pts.ds)
    u = Vector{ComplexF64}(undef, ws.dim)
    sig = Ref{Float64}(0)
    GC.@preserve ds u qbg_check(ccall((:qbg_solve_vect, libqbgpu), Int32,
        (Ptr{Cvoid}, Float64, Ptr{Float64}, Ref{Float64}, Ptr{ComplexF64}), ws.h, k, ds, sig, u))
    return sig[], u
end

end # module
