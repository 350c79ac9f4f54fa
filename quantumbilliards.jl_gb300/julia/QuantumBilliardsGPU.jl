# QuantumBilliardsGPU.jl — Julia binding of libqbgpu (ccall shim).
#
# Adds GPU methods to QuantumBilliards.jl's own functions for a wrapper solver
# type, so existing driver code (k_sweep, compute_spectrum_beyn, EBIM) keeps
# its signatures:
#   construct_matrices!                          (dlp_kress.jl:1627-1679, cfie_kress.jl:893-929)
#   construct_boundary_matrices!                 (chebyshev_euclidian_helmholtz_{dlp,cfie}_kress.jl:1110, 1431)
#   construct_boundary_matrices_with_derivatives! (..._dlp_kress.jl:1126-1144, ..._cfie_kress.jl:1507-1573)
#   construct_B_matrix                           (beyn.jl:257-322) through qbg_beyn_B
#   solve(solver, basis, pts[, ws], k; which=:svd), k_sweep (dlp_kress.jl:1783-1820, sweepmethods.jl:132-152)
# One device workspace is kept per (solver, discretisation) and reused by every
# call; methods take the reference's own workspace objects in the place where
# it passes them and look the device workspace up by the discretisation.
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

# symmetry orbits in the library's 0-based layout: DLP from the reference's
# periodic index orbits (symmetry.jl:214-261), CFIE from its reduced workspace
# (cfie_kress.jl:264-289); nothing without a symmetry
function _reduction(inner, pts)
    isnothing(inner.symmetry) && return nothing
    if _form(inner) == QBG_FORM_DLP
        p = pts isa AbstractVector ? pts[1] : pts
        rws = QB.build_dlp_kress_workspace(inner, p)
        Ifund, f2f, f2s = rws.Ifund, rws.fund_to_full, rws.fund_to_scale
    else
        ws = QB.build_cfie_kress_workspace(inner, pts isa AbstractVector ? pts : [pts])
        Ifund, f2f, f2s = ws.Ifund, ws.fund_to_full, ws.fund_to_scale
    end
    m, norb = length(Ifund), length(f2f[1])
    fund = Int64.(Ifund .- 1)
    orbit = Int64[f2f[b][l] - 1 for l in 1:norb, b in 1:m]        # orbit b's members contiguous
    scale = Float64[]
    for b in 1:m, l in 1:norb
        push!(scale, real(f2s[b][l]), imag(f2s[b][l]))
    end
    return fund, vec(orbit), scale, norb
end

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
    red = _reduction(solver.inner, pts)
    fund, orbit, scale, norb = red === nothing ? (Int64[], Int64[], Float64[], 0) : red
    keep = Any[offs, x, y, dx, dy, ddx, ddy, ts, wsv, fund, orbit, scale]
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve keep begin
        d = QbgGeomDesc(_form(solver.inner), Int32(length(comps)), pointer(offs), pointer(x), pointer(y),
                        pointer(dx), pointer(dy), pointer(ddx), pointer(ddy), pointer(ts), pointer(wsv),
                        Int64(length(fund)), Int32(norb),
                        isempty(fund) ? C_NULL : pointer(fund), isempty(orbit) ? C_NULL : pointer(orbit),
                        isempty(scale) ? C_NULL : pointer(scale),
                        0, 0, 0, 0, C_NULL, C_NULL, C_NULL, C_NULL)  # Kress; an Alpert solver fills the cache fields
        qbg_check(ccall((:qbg_geom_create, libqbgpu), Int32, (Ref{QbgGeomDesc}, Ref{Ptr{Cvoid}}), d, h))
    end
    dim = Ref{Int64}(0)
    qbg_check(ccall((:qbg_geom_dim, libqbgpu), Int32, (Ptr{Cvoid}, Ref{Int64}), h[], dim))
    return GPUWorkspace(h[], Int(dim[]), keep)
end

# one device workspace per (solver, discretisation), reused by every call
const _WS_CACHE = IdDict{Any,Any}()
function cached_workspace(solver::GPUSolver, pts)
    inner = get!(IdDict{Any,Any}, _WS_CACHE, solver)
    return get!(() -> gpu_workspace(solver, pts), inner, pts)
end
_ws(solver::GPUSolver, pts, ws::GPUWorkspace) = ws
_ws(solver::GPUSolver, pts, ws) = cached_workspace(solver, pts)   # the reference's own workspace types

# outs: [A(z_1)...A(z_n)] (+ [A'...], [A''...]) in place, direct or through Chebyshev panels
function _assemble!(ws::GPUWorkspace, zj, outs::Vector{Matrix{ComplexF64}}, deriv::Bool, use_chebyshev::Bool,
                    n_panels_h::Int, M_h::Int, n_panels_j::Int, M_j::Int)
    ks = ComplexF64.(collect(zj))
    ptrs = [pointer(T) for T in outs]
    GC.@preserve outs ks begin
        if use_chebyshev
            prm = QbgChebParams(Int32(n_panels_h), Int32(M_h), Int32(n_panels_j), Int32(M_j))
            qbg_check(ccall((:qbg_assemble_cheb, libqbgpu), Int32,
                (Ptr{Cvoid}, Ptr{ComplexF64}, Int64, Int32, Int32, Int32, Ref{QbgChebParams}, Ptr{Ptr{ComplexF64}}),
                ws.h, ks, length(ks), deriv ? 1 : 0, QBG_PREC_FP64, 0, prm, ptrs))
        else
            qbg_check(ccall((:qbg_assemble, libqbgpu), Int32,
                (Ptr{Cvoid}, Ptr{ComplexF64}, Int64, Int32, Int32, Int32, Ptr{Ptr{ComplexF64}}),
                ws.h, ks, length(ks), deriv ? 1 : 0, QBG_PREC_FP64, 0, ptrs))
        end
    end
    return nothing
end

# construct_boundary_matrices!(Tbufs, solver, pts, zj; use_chebyshev, panels...) — complex k, multi-k
function QB.construct_boundary_matrices!(Tbufs::Vector{Matrix{ComplexF64}}, solver::GPUSolver, pts,
                                         zj::AbstractVector{ComplexF64}; use_chebyshev::Bool=true,
                                         n_panels_h::Int=15000, M_h::Int=5, n_panels_j::Int=3000, M_j::Int=5,
                                         kwargs...)
    _assemble!(cached_workspace(solver, pts), zj, Tbufs, false, use_chebyshev, n_panels_h, M_h, n_panels_j, M_j)
    return nothing
end

# construct_boundary_matrices_with_derivatives!(Tbufs, dTbufs, ddTbufs, solver, pts, zj; ...)
function QB.construct_boundary_matrices_with_derivatives!(Tbufs::Vector{Matrix{ComplexF64}},
                                                          dTbufs::Vector{Matrix{ComplexF64}},
                                                          ddTbufs::Vector{Matrix{ComplexF64}}, solver::GPUSolver,
                                                          pts, zj::AbstractVector{ComplexF64};
                                                          use_chebyshev::Bool=true, n_panels_h::Int=15000,
                                                          M_h::Int=5, n_panels_j::Int=3000, M_j::Int=5, kwargs...)
    outs = vcat(Tbufs, dTbufs, ddTbufs)
    _assemble!(cached_workspace(solver, pts), zj, outs, true, use_chebyshev, n_panels_h, M_h, n_panels_j, M_j)
    return nothing
end

# construct_matrices!(solver, A[, dA, ddA], pts, ws, k) — real k (sweep, EBIM, Newton); ws may be the
# reference's workspace (DLPKressWorkspace, DLPKressReducedWorkspace, CFIEKressWorkspace) or a GPUWorkspace
function QB.construct_matrices!(solver::GPUSolver, A::Matrix{ComplexF64}, dA::Matrix{ComplexF64},
                                ddA::Matrix{ComplexF64}, pts, ws, k::Real; kwargs...)
    _assemble!(_ws(solver, pts, ws), [complex(k)], [A, dA, ddA], true, false, 0, 0, 0, 0)
    return A, dA, ddA
end
function QB.construct_matrices!(solver::GPUSolver, A::Matrix{ComplexF64}, pts, ws, k::Real; kwargs...)
    _assemble!(_ws(solver, pts, ws), [complex(k)], [A], false, false, 0, 0, 0, 0)
    return A
end

# sigma_min over a k list on the device (qbg_sigma_min: batched LU, inverses, subspace iteration)
function gpu_sigma_min(ws::GPUWorkspace, ks::AbstractVector{<:Real})
    kk = Float64.(collect(ks))
    sig = Vector{Float64}(undef, length(kk))
    GC.@preserve kk sig qbg_check(ccall((:qbg_sigma_min, libqbgpu), Int32,
        (Ptr{Cvoid}, Ptr{Float64}, Int64, Ptr{Float64}), ws.h, kk, length(kk), sig))
    return sig
end

# solve(solver, basis, pts[, ws][, A], k; which=:svd) (dlp_kress.jl:1783-1820): sigma_min(A(k))
function _solve_svd(solver::GPUSolver, pts, ws, k, which)
    which === :svd || error("qbgpu: solve on the GPU computes which=:svd (sigma_min), not $(which)")
    return gpu_sigma_min(_ws(solver, pts, ws), [k])[1]
end
QB.solve(solver::GPUSolver, basis::QB.AbsBasis, pts, k::Real; which::Symbol=:svd, kwargs...) =
    _solve_svd(solver, pts, nothing, k, which)
QB.solve(solver::GPUSolver, basis::QB.AbsBasis, pts, ws, k::Real; which::Symbol=:svd, kwargs...) =
    _solve_svd(solver, pts, ws, k, which)
QB.solve(solver::GPUSolver, basis::QB.AbsBasis, A::AbstractMatrix, pts, ws, k::Real; which::Symbol=:svd, kwargs...) =
    _solve_svd(solver, pts, ws, k, which)

# k_sweep(solver, basis, billiard, ks; which=:svd) (sweepmethods.jl:132-152): the discretisation at
# maximum(ks) (sweepmethods.jl:51-60), every sigma_min in one batched device call
function QB.k_sweep(solver::GPUSolver, basis::QB.AbsBasis, billiard::QB.AbsBilliard, ks; which::Symbol=:svd,
                    kwargs...)
    which === :svd || error("qbgpu: k_sweep on the GPU computes which=:svd (sigma_min)")
    pts = QB.evaluate_points(solver.inner, billiard, maximum(ks))
    return gpu_sigma_min(cached_workspace(solver, pts), ks)
end

# construct_B_matrix(solver, pts, N, k0, R; nq, r, svd_tol, rng, use_chebyshev, panels) — beyn.jl:257-322
# through qbg_beyn_B: the assembly, LU, solves, moments, the thin SVD (device QR of A0, Jacobi SVD of
# its R), the absolute rank test and B in the library; the regrowth draws a fresh N x 2r block from
# rng after the first block saturates, and the loop is left after that one pass (beyn.jl:291-309).
function QB.construct_B_matrix(solver::GPUSolver, pts, N::Int, k0::Complex{Float64}, R::Float64;
                               nq::Int=64, r::Int=48, svd_tol=1e-14, rng=QB.MersenneTwister(0),
                               use_chebyshev::Bool=true, n_panels_h::Int=15000, M_h::Int=5, n_panels_j::Int=3000,
                               M_j::Int=5, kwargs...)
    ws = cached_workspace(solver, pts)
    @assert ws.dim == N
    h = Ref{Ptr{Cvoid}}(C_NULL)
    opts = QbgBeynOpts(0, 10, 1e-6, 0, use_chebyshev ? 0 : 1,
                       QbgChebParams(Int32(n_panels_h), Int32(M_h), Int32(n_panels_j), Int32(M_j)), 0, 0, 0, 0)
    qbg_check(ccall((:qbg_beyn_create, libqbgpu), Int32,
        (Ptr{Cvoid}, Float64, Float64, Float64, Int32, Int32, Ref{QbgBeynOpts}, Ref{Ptr{Cvoid}}),
        ws.h, real(k0), imag(k0), R, nq, solver.prec, opts, h))
    Bcall(V) = begin
        c = size(V, 2)
        B = Vector{ComplexF64}(undef, c * c); U = Matrix{ComplexF64}(undef, N, c)
        rk = Ref{Int64}(0); rused = Ref{Int64}(0)
        GC.@preserve V B U qbg_check(ccall((:qbg_beyn_B, libqbgpu), Int32,
            (Ptr{Cvoid}, Ptr{ComplexF64}, Int64, Ptr{ComplexF64}, Float64, Ptr{ComplexF64}, Ptr{ComplexF64},
             Ptr{Float64}, Ref{Int64}, Ref{Int64}, Ptr{Cvoid}),
            h[], V, c, C_NULL, svd_tol, B, U, C_NULL, rk, rused, C_NULL))
        k = Int(rk[])
        reshape(B[1:k*k], k, k), U[:, 1:k], k
    end
    try
        V = randn(rng, ComplexF64, N, r)
        B, Uk, rk = Bcall(V)
        rk == 0 && return Matrix{ComplexF64}(undef, N, 0), Matrix{ComplexF64}(undef, N, 0)
        if rk == r && 2r < N
            B, Uk, rk = Bcall(randn(rng, ComplexF64, N, 2r))
        end
        return B, Uk
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
    QB.construct_matrices!(solver, A, dA, ddA, pts, cached_workspace(solver, pts), k)
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
                                     pts, ws, k::Real; kwargs...)
    ds = collect(Float64, pts.ds)
    g = _ws(solver, pts, ws)
    GC.@preserve A ds qbg_check(ccall((:qbg_adjoint_fredholm, libqbgpu), Int32,
        (Ptr{Cvoid}, Float64, Ptr{Float64}, Ptr{ComplexF64}, Int32), g.h, k, ds, A, Int32(0)))
    return A
end
function QB.solve_vect(solver::GPUSolver, basis::QB.AbsBasis, pts, ws, k::Real; kwargs...)
    ds = collect(Float64, pts.ds)
    g = _ws(solver, pts, ws)
    u = Vector{ComplexF64}(undef, g.dim)
    sig = Ref{Float64}(0)
    GC.@preserve ds u qbg_check(ccall((:qbg_solve_vect, libqbgpu), Int32,
        (Ptr{Cvoid}, Float64, Ptr{Float64}, Ref{Float64}, Ptr{ComplexF64}), g.h, k, ds, sig, u))
    return sig[], u
end

end # module
