"""
    PTDiffusion

Julia host side of the GB300 accelerated pseudo-transient diffusion library
(libptd.so, C ABI in include/ptd.h).  It keeps the reference scripts' driver
interface: `diffusion_2D_(; nx, ny, ...)` builds the grid and H0 exactly as
scripts/diff_2D_nonlin.jl:46-74 does, hands the PT solve to the library via
`ccall`, and returns `(xc, yc, H)` like the script's `USE_RETURN=true` branch
(scripts/diff_2D_nonlin.jl:105,108-112), plus the iteration counts and the
residual history.

Not executed in this repository's test suite (no Julia toolchain on the build
or GPU hosts); the Python binding in ptdiff/ calls the same entry points and
is what the tests exercise.
"""
module PTDiffusion

export PtdParams, diffusion_1D_, diffusion_2D_, diffusion_3D_, diffusion_react_1D_, diffusion_react_2D_,
       solve!, AdjointSolver, misfit, forward!, gradient!

const libptd = joinpath(@__DIR__, "..", "..", "libptd.so")

const PTD_OK = Cint(0)
const MODEL = Dict(:lin => Int32(0), :linstep => Int32(1), :nonlin => Int32(2))
const PRECISION = Dict(:fp64 => Int32(0), :fp32_dc => Int32(1), :df64 => Int32(2), :dfh => Int32(3),
                       :fp32_rb => Int32(4))

# Mirror of `ptd_params` (include/ptd.h); field order and types must match.
mutable struct PtdParams
    ndim::Int32; model::Int32
    nx::Int32; ny::Int32; nz::Int32
    lx::Float64; ly::Float64; lz::Float64
    dt::Float64
    nt::Int32; itmax::Int32; nchk::Int32; precision::Int32
    tol::Float64; cfl::Float64; resc::Float64; D::Float64
    resid_mode::Int32; norm::Int32
    norm_len::Float64
    flags::Int32; dc_max_outer::Int32
    dc_inner_rtol::Float64
    reserved::NTuple{8,Int32}
end

function PtdParams(ndim::Integer, model::Symbol)
    p = PtdParams(zeros(Int32, 5)..., zeros(4)..., zeros(Int32, 4)..., zeros(4)..., Int32(0), Int32(0),
                  0.0, Int32(0), Int32(0), 0.0, ntuple(_ -> Int32(0), 8))
    st = ccall((:ptd_params_init, libptd), Cint, (Ref{PtdParams}, Int32, Int32), p, Int32(ndim), MODEL[model])
    st == PTD_OK || error(ptd_error("ptd_params_init", st))
    return p
end

function ptd_error(where, st)
    msg = unsafe_string(ccall((:ptd_strerror, libptd), Cstring, (Cint,), st))
    detail = unsafe_string(ccall((:ptd_last_error, libptd), Cstring, ()))
    return "$where: $msg ($detail)"
end

"""
    solve!(p, H; D=nothing) -> (iters_per_step, errhist)

Solve `p.nt` physical steps in place on `H` (Float64, x fastest; host Array or
a CuArray's device pointer).  Throws on NaN like the reference's
`error("NaN")` (scripts/diff_2D_nonlin.jl:90).
"""
function solve!(p::PtdParams, H::AbstractArray{Float64}; D=nothing, errcap::Integer=100_000)
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:ptd_create, libptd), Cint, (Ref{Ptr{Cvoid}}, Ref{PtdParams}), ctx, p)
    st == PTD_OK || error(ptd_error("ptd_create", st))
    iters = zeros(Int32, max(p.nt, 1))
    errs = zeros(Float64, errcap)
    nerr = Ref{Int32}(0)
    try
        Dptr = D === nothing ? Ptr{Float64}(C_NULL) : pointer(D)
        st = ccall((:ptd_solve, libptd), Cint,
                   (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}, Ptr{Float64}, Int32, Ref{Int32}),
                   ctx[], pointer(H), Dptr, iters, errs, Int32(errcap), nerr)
        st == PTD_OK || error(st == 2 ? "NaN" : ptd_error("ptd_solve", st))
    finally
        ccall((:ptd_destroy, libptd), Cvoid, (Ptr{Cvoid},), ctx[])
    end
    return iters[1:p.nt], errs[1:min(nerr[], errcap)]
end

"""
    solve_react!(p, H, Heq) -> iters

The reaction scripts' single PT loop (scripts/diff_1D_react.jl:45-66,
diff_2D_react.jl:55-72): H from zero towards Heq with theta_kin in place of
dt, i.e. one implicit step of the linear solver with Hold = Heq
(`ptd_set_state2`).
"""
function solve_react!(p::PtdParams, H::AbstractArray{Float64}, Heq::AbstractArray{Float64})
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:ptd_create, libptd), Cint, (Ref{Ptr{Cvoid}}, Ref{PtdParams}), ctx, p)
    st == PTD_OK || error(ptd_error("ptd_create", st))
    iters = zeros(Int32, 1)
    try
        st = ccall((:ptd_set_state2, libptd), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                   ctx[], pointer(H), pointer(Heq), C_NULL)
        st == PTD_OK || error(ptd_error("ptd_set_state2", st))
        st = ccall((:ptd_step, libptd), Cint, (Ptr{Cvoid}, Int32, Ptr{Int32}, Ptr{Float64}, Int32, Ptr{Int32}),
                   ctx[], Int32(1), iters, C_NULL, Int32(0), C_NULL)
        st == PTD_OK || error(st == 2 ? "NaN" : ptd_error("ptd_step", st))
        st = ccall((:ptd_get_state, libptd), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx[], pointer(H))
        st == PTD_OK || error(ptd_error("ptd_get_state", st))
    finally
        ccall((:ptd_destroy, libptd), Cvoid, (Ptr{Cvoid},), ctx[])
    end
    return iters[1]
end

# Julia's LinRange cell centres, as in the scripts (e.g. scripts/diff_2D_nonlin.jl:63).
cell_centres(l, n) = LinRange(l / n / 2, l - l / n / 2, n)

function diffusion_1D_(; model::Symbol=:lin, nx::Integer=parse(Int, get(ENV, "NX", "512")),
                       precision::Symbol=:fp64)
    p = PtdParams(1, model); p.nx = nx; p.precision = PRECISION[precision]
    lx = p.lx; xc = cell_centres(lx, nx)
    H = Array(exp.(-(xc .- lx / 2) .^ 2))
    D = nothing
    if model == :linstep
        D = ones(nx); D[1:Int(ceil(nx / 2.2))] .= 1e-4          # scripts/diff_1D_linstep.jl:69-70
        p.D = 1.0
    end
    iters, errs = solve!(p, H; D=D)
    return xc, H, iters, errs
end

function diffusion_2D_(; model::Symbol=:nonlin, nx::Integer=parse(Int, get(ENV, "NX", "512")),
                       ny::Integer=parse(Int, get(ENV, "NY", "512")), precision::Symbol=:fp64)
    p = PtdParams(2, model); p.nx = nx; p.ny = ny; p.precision = PRECISION[precision]
    lx, ly = p.lx, p.ly
    xc, yc = cell_centres(lx, nx), cell_centres(ly, ny)
    H = Array(exp.(-(xc .- lx / 2) .^ 2 .- ((yc .- ly / 2)') .^ 2))  # scripts/diff_2D_nonlin.jl:71
    D = nothing
    if model == :linstep                                          # scripts/diff_2D_linstep.jl:81-83
        D = ones(nx, ny); D[1:Int(ceil(nx / 2.2)), :] .= 1e-4; D[:, 1:Int(ceil(ny / 2.2))] .= 1e-4
    end
    iters, errs = solve!(p, H; D=D)
    return xc, yc, H, iters, errs
end

function diffusion_3D_(; model::Symbol=:nonlin, nx::Integer=parse(Int, get(ENV, "NX", "64")),
                       ny::Integer=parse(Int, get(ENV, "NY", "64")), nz::Integer=parse(Int, get(ENV, "NZ", "64")),
                       precision::Symbol=:fp64)
    p = PtdParams(3, model); p.nx = nx; p.ny = ny; p.nz = nz; p.precision = PRECISION[precision]
    lx, ly, lz = p.lx, p.ly, p.lz
    dx, dy, dz = lx / nx, ly / ny, lz / nz
    # ImplicitGlobalGrid coordinates on one rank: x_g(ix) = (ix-1)*dx
    # (scripts/diff_3D/diff_3D_nonlin_multixpu.jl:86)
    H = [exp(-((ix - 1) * dx - 0.5lx + dx / 2)^2 - ((iy - 1) * dy - 0.5ly + dy / 2)^2 -
             ((iz - 1) * dz - 0.5lz + dz / 2)^2) for ix = 1:nx, iy = 1:ny, iz = 1:nz]
    D = nothing
    if model == :linstep                                          # diff_3D_linstep_multixpu.jl:99-104
        D = ones(nx, ny, nz)
        D[[(ix - 1) * dx < lx / 2.2 for ix = 1:nx], :, :] .= 1e-4
        D[:, [(iy - 1) * dy < ly / 2.2 for iy = 1:ny], :] .= 1e-4
    end
    iters, errs = solve!(p, H; D=D)
    return cell_centres(lx, nx), cell_centres(ly, ny), cell_centres(lz, nz), H, iters, errs
end

# Reaction-diffusion drivers (scripts/diff_1D_react.jl:31-47, diff_2D_react.jl:33-58):
# D = 1, theta_kin = 0.1 (the dt of the equivalent implicit step), H0 = Heq a
# Gaussian, H starting at zero.
function diffusion_react_1D_(; nx::Integer=parse(Int, get(ENV, "NX", "512")), precision::Symbol=:fp64)
    p = PtdParams(1, :lin); p.nx = nx; p.lx = 20.0; p.dt = 0.1; p.nt = 1; p.cfl = 0.99
    p.precision = PRECISION[precision]
    xc = cell_centres(p.lx, nx)
    Heq = Array(exp.(-(xc .- p.lx / 2) .^ 2))
    H = zeros(nx)
    iters = solve_react!(p, H, Heq)
    return xc, H, iters
end

function diffusion_react_2D_(; nx::Integer=parse(Int, get(ENV, "NX", "512")),
                             ny::Integer=parse(Int, get(ENV, "NY", "512")), precision::Symbol=:fp64)
    p = PtdParams(2, :lin); p.nx = nx; p.ny = ny; p.dt = 0.1; p.nt = 1
    p.precision = PRECISION[precision]
    xc, yc = cell_centres(p.lx, nx), cell_centres(p.ly, ny)
    Heq = Array(exp.(-(xc .- p.lx / 2) .^ 2 .- ((yc .- p.ly / 2)') .^ 2))
    H = zeros(nx, ny)
    iters = solve_react!(p, H, Heq)
    return xc, yc, H, iters
end

# ---------------------------------------------------------------------------
# Adjoint (no reference counterpart): gradient of L = 1/2 sum_inner (H^nt - Ht)^2
# with respect to the log-coefficient m (D = exp(m) H^3) and H0, through
# ptd_adj_* (one FP64 checkpoint per physical step).

mutable struct AdjointSolver
    h::Ptr{Cvoid}
    p::PtdParams
end

function AdjointSolver(p::PtdParams)
    h = Ref{Ptr{Cvoid}}(C_NULL)
    st = ccall((:ptd_adj_create, libptd), Cint, (Ref{Ptr{Cvoid}}, Ref{PtdParams}), h, p)
    st == PTD_OK || error(ptd_error("ptd_adj_create", st))
    a = AdjointSolver(h[], p)
    finalizer(x -> ccall((:ptd_adj_destroy, libptd), Cvoid, (Ptr{Cvoid},), x.h), a)
    return a
end

function forward!(a::AdjointSolver, H0, m, Ht)
    loss = Ref{Float64}(0.0)
    iters = zeros(Int32, max(a.p.nt, 1))
    st = ccall((:ptd_adj_forward, libptd), Cint,
               (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ref{Float64}, Ptr{Float64}, Ptr{Int32}),
               a.h, pointer(H0), pointer(m), pointer(Ht), loss, C_NULL, iters)
    st == PTD_OK || error(ptd_error("ptd_adj_forward", st))
    return loss[]
end

function gradient!(a::AdjointSolver)
    gm, gh = zeros(a.p.nx, a.p.ny, a.p.nz), zeros(a.p.nx, a.p.ny, a.p.nz)
    iters = zeros(Int32, max(a.p.nt, 1))
    st = ccall((:ptd_adj_gradient, libptd), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Int32}),
               a.h, pointer(gm), pointer(gh), iters)
    st == PTD_OK || error(ptd_error("ptd_adj_gradient", st))
    return gm, gh
end

"""
    misfit(a, m, H0, Ht) -> L

L2 misfit of the final state; differentiable through the ChainRulesCore
`rrule` below (the Julia counterpart of ptdiff.misfit_function()).
"""
misfit(a::AdjointSolver, m, H0, Ht) = forward!(a, H0, m, Ht)

# The ChainRulesCore rrule of `misfit` is the package extension
# ext/PTDiffusionChainRulesCoreExt.jl (ChainRulesCore is a weak dependency:
# Julia loads the extension whenever both packages are loaded, in any order).

end # module
