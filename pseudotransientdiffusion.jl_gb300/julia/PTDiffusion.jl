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

export PtdParams, diffusion_1D_, diffusion_2D_, diffusion_3D_, solve!

const libptd = joinpath(@__DIR__, "..", "libptd.so")

const PTD_OK = Cint(0)
const MODEL = Dict(:lin => Int32(0), :linstep => Int32(1), :nonlin => Int32(2))
const PRECISION = Dict(:fp64 => Int32(0), :fp32_dc => Int32(1))

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

end # module
