"""
    GPUCellListSPH_GB300

Drop-in binding of GPUCellListSPH.jl's public API (src/GPUCellListSPH.jl:9-17)
over `libgcsph.so`, the sm_103a CUDA library whose C ABI is
`include/gcsph.h`.  Types, field names, constructors and function names are the
reference's; every computation runs in the library, called through `ccall` on
the caller's `CuArray`s (device pointers, no copies) and CUDA.jl's task-local
stream.  Float64 only, as the library computes in FP64.

Differences from the reference's structs, each because the library keeps the
data in its own sorted layout:
  * `GPUCellList.pcell` and `.celllist` are empty arrays: the library holds
    cell membership as a sort, not as a dense `mppcell x CELL` array;
  * `SPHProblem.W` and `.∇W` are empty: the pair values are fused into the
    pair sums and never stored;
  * the other work arrays (`P`, `∑∂v∂t`, `∑∂ρ∂t`, `ρΔt½`, `vΔt½`, `xΔt½`,
    `cΔx`, `∑W`, `∑∇W`, `buf2`) are refreshed from the library when read,
    and the scalar fields are pushed to it when assigned.

The library's path defaults to the in-tree build; set `ENV["GCSPH_LIB"]`
before loading this module to use another copy.
"""
module GPUCellListSPH_GB300

using CUDA

export GPUCellList, update!, partialupdate!, neighborlist, neighborlistview
export SPHProblem, stepsolve!, timesolve!, get_points, get_velocity, get_density, get_pressure, get_acceleration
export get_dpccorr, get_simtime, get_dt, get_sumw, get_sumgradw, get_ptype
export sphW!, sph∇W!, sph∑W!, sph∑∇W!, ∂ρ∂tDDT!, pressure!, ∂v∂t!, ∂v∂t_av!, ∂v∂t_visc!, ∂v∂t_addgrav!, ∂v∂tpF!,
       dpcreg!, cspmcorr!, xsphcorr!, fbmolforce!

const libgcsph = get(ENV, "GCSPH_LIB", joinpath(@__DIR__, "..", "_build", "libgcsph.so"))

const GCSPH_OK = 0
const GCSPH_ECAPACITY = 2

struct GcsphError <: Exception
    code::Int
    msg::String
end
Base.showerror(io::IO, e::GcsphError) = print(io, "gcsph error ", e.code, ": ", e.msg)

lasterror() = unsafe_string(ccall((:gcsph_last_error, libgcsph), Cstring, ()))
check(rc::Integer, allow = ()) = (rc == GCSPH_OK || rc in allow) ? Int(rc) : throw(GcsphError(rc, lasterror()))

# device address of a CuArray, and a host array of D of them (the layout of
# `const double* const*` and of the reference's NTuple{D, CuArray})
devaddr(a::CuArray) = reinterpret(UInt64, pointer(a))
devaddrs(v) = Ref(ntuple(i -> devaddr(v[i]), length(v)))
stream() = CUDA.stream().handle

# ---------------------------------------------------------------- cell list

"""
    GPUCellList{T, D}

Fields as in src/celllist.jl:1-15, plus the library handle.
"""
mutable struct GPUCellList{T <: AbstractFloat, D}
    n::Int
    dist::T
    cs::Tuple{Vararg{T}}
    offset::Tuple{Vararg{T}}
    grid::Tuple{Vararg{Int}}
    points::NTuple{D, CuArray{T}}
    pcell::CuArray{NTuple{D, Int32}}
    cellpnum::CuArray{Int32}
    cnt::CuArray
    celllist::CuArray{Int32}
    pairs::CuArray{Tuple{Int32, Int32}}
    pairsn::Int
    handle::Ptr{Cvoid}
end

"""
    GPUCellList(points, cellsize, dist; MIN = nothing, MAX = nothing, mppcell = 0, mpairs = 0)

src/celllist.jl:22-88 -- `gcl_create`, then the constructor's capacity
policy on `gcl_maxpairs` and `gcl_emit_pairs`.
"""
function GPUCellList(points::NTuple{D, AbstractArray{T}}, cellsize, dist; MIN = nothing, MAX = nothing,
                     mppcell = 0, mpairs = 0) where {T <: AbstractFloat, D}
    pl = length.(points)
    if !all(x -> x == first(pl), pl) error("length of points not equal") end
    if D < 2 || D > 3 error("wrong dimention") end
    T === Float64 || error("libgcsph computes in Float64: pass Float64 points")
    dist = T(dist)
    cellsize = T.(Tuple(cellsize))
    for i in eachindex(cellsize)
        if cellsize[i] < dist
            @warn "Cell size (dim $i) < dist, cell size set equal dist"
            cellsize = Base.setindex(cellsize, dist, i)
        end
    end
    N = first(pl)
    pts = Tuple(CuArray{T}(p) for p in points)
    mn = isnothing(MIN) ? C_NULL : Ref(Float64.(Tuple(MIN)))
    mx = isnothing(MAX) ? C_NULL : Ref(Float64.(Tuple(MAX)))
    h = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve pts check(ccall((:gcl_create, libgcsph), Cint,
        (Int32, Int64, Ptr{UInt64}, Ptr{Float64}, Float64, Ptr{Float64}, Ptr{Float64}, Ptr{Cvoid}, Ptr{Ptr{Cvoid}}),
        D, N, devaddrs(pts), Ref(Float64.(cellsize)), dist, mn, mx, stream(), h))
    cs, off, cell = Ref(ntuple(_ -> 0.0, 3)), Ref(ntuple(_ -> 0.0, 3)), Ref(ntuple(_ -> Int64(0), 3))
    check(ccall((:gcl_grid, libgcsph), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Int64}), h[], cs, off, cell))
    grid = ntuple(i -> Int(cell[][i]), D)
    cellpnum = CUDA.zeros(Int32, grid...)
    check(ccall((:gcl_cellpnum, libgcsph), Cint, (Ptr{Cvoid}, UInt64), h[], devaddr(cellpnum)))
    # mppcell has no storage behind it here (no dense cell list); kept for the signature
    if mpairs == 0
        mp = Ref{Int64}(0)
        check(ccall((:gcl_maxpairs, libgcsph), Cint, (Ptr{Cvoid}, Ptr{Int64}), h[], mp))
        mpairs = Int(mp[])
    end
    c = GPUCellList{T, D}(N, dist, ntuple(i -> T(cs[][i]), D), ntuple(i -> T(off[][i]), D), grid, pts,
                          CuArray{NTuple{D, Int32}}(undef, 0), cellpnum, CUDA.zeros(Int32, 1),
                          CUDA.zeros(Int32, 0), CUDA.fill((zero(Int32), zero(Int32)), mpairs), 0, h[])
    finalizer(c) do x
        x.handle == C_NULL || ccall((:gcl_destroy, libgcsph), Cvoid, (Ptr{Cvoid},), x.handle)
        x.handle = C_NULL
    end
    total_pairs = emit!(c, true)                                    # src/celllist.jl:76-86
    if total_pairs > mpairs
        @warn "List of pairs not full, call `update!(c::GPUCellList)` to extend pair list!"
    end
    if total_pairs < mpairs * 0.8
        new_pairs = CUDA.fill((zero(Int32), zero(Int32)), Int(ceil(total_pairs / 0.8)))
        copyto!(new_pairs, view(c.pairs, 1:length(new_pairs)))
        CUDA.unsafe_free!(c.pairs)
        c.pairs = new_pairs
    end
    c.pairsn = total_pairs
    c
end

# write the pair set of the last build into c.pairs (the first length(c.pairs)
# pairs when it does not fit); the full count either way
function emit!(c::GPUCellList, fillzero::Bool)
    n = Ref{Int64}(0)
    check(ccall((:gcl_emit_pairs, libgcsph), Cint, (Ptr{Cvoid}, UInt64, Int64, Cint, Ptr{Int64}),
                c.handle, length(c.pairs) == 0 ? UInt64(0) : devaddr(c.pairs), length(c.pairs), fillzero, n),
          (GCSPH_ECAPACITY,))
    Int(n[])
end

function refresh_cellpnum!(c::GPUCellList)
    check(ccall((:gcl_cellpnum, libgcsph), Cint, (Ptr{Cvoid}, UInt64), c.handle, devaddr(c.cellpnum)))
end

# the capacity policy of update!, src/celllist.jl:117-133, on a new total
function apply_update_policy!(c::GPUCellList, total::Int, fillzero::Bool)
    realloc = false
    cap = length(c.pairs)
    if c.pairsn > cap || c.pairsn < cap * 0.6
        cap, realloc = Int(ceil(c.pairsn / 0.8)), true
    end
    if total > cap
        cap, realloc = Int(ceil(total / 0.8)), true
    end
    if realloc
        CUDA.unsafe_free!(c.pairs)
        c.pairs = CUDA.fill((zero(Int32), zero(Int32)), cap)
    end
    emit!(c, fillzero || realloc)
    c.pairsn = total
end

"""
    update!(c::GPUCellList, fillzero::Bool = true)

src/celllist.jl:95-134 -- `gcl_update`: re-bin every point into the frozen
grid and rebuild the pair set.
"""
function update!(c::GPUCellList, fillzero::Bool = true)
    n = Ref{Int64}(0)
    check(ccall((:gcl_update, libgcsph), Cint, (Ptr{Cvoid}, Ptr{Int64}), c.handle, n))
    refresh_cellpnum!(c)
    apply_update_policy!(c, Int(n[]), fillzero)
end

"""
    partialupdate!(c::GPUCellList, fillzero::Bool = true)

src/celllist.jl:141-145 -- `gcl_partialupdate`: the pair search with the
cell membership of the last update! and the current coordinates.
"""
function partialupdate!(c::GPUCellList, fillzero::Bool = true)
    n = Ref{Int64}(0)
    check(ccall((:gcl_partialupdate, libgcsph), Cint, (Ptr{Cvoid}, Ptr{Int64}), c.handle, n))
    emit!(c, fillzero)
    c.pairsn = Int(n[])
end

neighborlist(c::GPUCellList) = c.pairs                        # src/celllist.jl:152-154
neighborlistview(c::GPUCellList) = view(c.pairs, 1:c.pairsn)  # src/celllist.jl:161-163

# ---------------------------------------------------------------- SPH problem

# gcsph_params, field order of include/gcsph.h
struct GcsphParams
    dx::Cdouble; h::Cdouble; H::Cdouble; rho0::Cdouble; m0::Cdouble; dt::Cdouble; alpha::Cdouble
    nu::Cdouble; g::Cdouble; c0::Cdouble; s::Cdouble; delta::Cdouble; CFL::Cdouble; nui::Cdouble
    etime::Cdouble; dpc_l0::Cdouble; dpc_pmin::Cdouble; dpc_pmax::Cdouble; dpc_lambda::Cdouble
    xsph_eps::Cdouble; bound_D::Cdouble; bound_l::Cdouble; gamma::Int32; cspmn::Int32
end

"""
    SPHProblem{T, D}

Fields as in src/sphproblem.jl:62-112, plus the library handle and the
Int32 copy of `ptype` the library reads.
"""
mutable struct SPHProblem{T, D}
    system::GPUCellList
    dim::Int
    dx::T
    h::T
    h⁻¹::T
    H::T
    H⁻¹::T
    sphkernel::Any
    ∑W::CuArray
    ∑∇W
    W::CuArray
    ∇W
    ∑∂v∂t
    ∑∂ρ∂t
    ρ::CuArray
    ρΔt½::CuArray
    v
    vΔt½
    xΔt½
    P::CuArray
    ptype::CuArray
    ρ₀::T
    m₀::T
    Δt::T
    α::T
    𝜈::T
    g::T
    c₀::T
    γ
    s::T
    δᵩ::T
    CFL::T
    buf::CuArray
    buf2
    etime::T
    cΔx
    nui::T
    dpc_l₀::T
    dpc_pmin::T
    dpc_pmax::T
    dpc_λ::T
    xsph_𝜀::T
    cspmn::Int
    bound_D::T
    bound_l::T
    handle::Ptr{Cvoid}
    ptype32::CuArray{Int32}
end

# the scalar fields the library keeps, and the library's field id of each
# work array (enum GCSPH_F_* in include/gcsph.h)
const SCALARS = (:dx, :h, :H, :ρ₀, :m₀, :Δt, :α, :𝜈, :g, :c₀, :s, :δᵩ, :CFL, :nui, :etime, :dpc_l₀, :dpc_pmin,
                 :dpc_pmax, :dpc_λ, :xsph_𝜀, :bound_D, :bound_l, :γ, :cspmn)
const WORKFIELDS = Dict(:P => 3, :∑∂v∂t => 4, :∑∂ρ∂t => 5, :ρΔt½ => 6, :vΔt½ => 7, :xΔt½ => 8, :cΔx => 9,
                        :∑W => 10, :∑∇W => 11, :buf2 => 12)

params(p::SPHProblem) = GcsphParams(
    getfield(p, :dx), getfield(p, :h), getfield(p, :H), getfield(p, :ρ₀), getfield(p, :m₀), getfield(p, :Δt),
    getfield(p, :α), getfield(p, :𝜈), getfield(p, :g), getfield(p, :c₀), getfield(p, :s), getfield(p, :δᵩ),
    getfield(p, :CFL), getfield(p, :nui), getfield(p, :etime), getfield(p, :dpc_l₀), getfield(p, :dpc_pmin),
    getfield(p, :dpc_pmax), getfield(p, :dpc_λ), getfield(p, :xsph_𝜀), getfield(p, :bound_D),
    getfield(p, :bound_l), Int32(getfield(p, :γ)), Int32(getfield(p, :cspmn)))

function push_params!(p::SPHProblem)
    check(ccall((:sph_set_params, libgcsph), Cint, (Ptr{Cvoid}, Ref{GcsphParams}), getfield(p, :handle), params(p)))
end

# the library advances etime and, with timestepping, Δt
function pull_params!(p::SPHProblem)
    r = Ref{GcsphParams}()
    check(ccall((:sph_get_params, libgcsph), Cint, (Ptr{Cvoid}, Ptr{GcsphParams}), getfield(p, :handle), r))
    setfield!(p, :etime, r[].etime)
    setfield!(p, :Δt, r[].dt)
end

function Base.setproperty!(p::SPHProblem, s::Symbol, x)
    v = setfield!(p, s, convert(fieldtype(typeof(p), s), x))
    s in SCALARS && getfield(p, :handle) != C_NULL && push_params!(p)
    v
end

function Base.getproperty(p::SPHProblem, s::Symbol)
    id = get(WORKFIELDS, s, -1)
    if id >= 0 && getfield(p, :handle) != C_NULL
        a = getfield(p, s)
        dst = a isa Tuple ? CUDA.zeros(Float64, getfield(p, :system).n * length(a)) : a
        check(ccall((:sph_get_field, libgcsph), Cint, (Ptr{Cvoid}, Int32, UInt64), getfield(p, :handle), id,
                    devaddr(dst)))
        if a isa Tuple                                        # D x N, dimension-major
            N = getfield(p, :system).n
            for d in eachindex(a)
                copyto!(a[d], 1, dst, (d - 1) * N + 1, N)
            end
        end
    end
    getfield(p, s)
end

"""
    SPHProblem(system, dx, h, H, sphkernel, ρ, ptype, ρ₀, m₀, Δt, α, c₀, γ, δᵩ, CFL; v = nothing, g = 9.81, s = 0.0)

src/sphproblem.jl:113-192 -- `sph_create` over the caller's ρ, v and ptype,
with the reference's defaults for the other fields (:172-191).
"""
function SPHProblem(system::GPUCellList{T, D}, dx, h, H, sphkernel, ρ, ptype, ρ₀, m₀, Δt, α, c₀, γ, δᵩ, CFL;
                    v = nothing, g = 9.81, s = 0.0) where {T <: AbstractFloat, D}
    N = system.n
    if isnothing(v) v = Tuple(CUDA.zeros(T, N) for n in 1:D) end
    if length(ρ) != N error("length(ρ) ($(length(ρ))) != N ($N)") end
    if length(ptype) != N error("length(ptype) ($(length(ptype))) != N ($N)") end
    if any(x -> length(x) != N, v) error("length(v) ($(length.(v))) != N ($N)") end
    z() = CUDA.zeros(T, N)
    zd() = Tuple(CUDA.zeros(T, N) for _ in 1:D)
    ptype32 = ptype isa CuArray{Int32} ? ptype : CuArray{Int32}(ptype)
    p = SPHProblem{T, D}(system, D, dx, h, 1 / h, H, 1 / H, sphkernel, z(), zd(), CUDA.zeros(T, 0),
                         Tuple(CUDA.zeros(T, 0) for _ in 1:D), zd(), z(), ρ, z(), v, zd(), zd(), z(), ptype,
                         ρ₀, m₀, Δt, α, 0.0, g, c₀, γ, s, δᵩ, CFL, z(), zd(), 0.0, zd(), system.dist - H,
                         0.0, 1.0, 10000.0, 0.01, 0.0, 15, 0.4, 2dx, C_NULL, ptype32)
    h_ = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:sph_create, libgcsph), Cint,
                (Ptr{Cvoid}, Ref{GcsphParams}, UInt64, Ptr{UInt64}, UInt64, Ptr{Ptr{Cvoid}}),
                system.handle, params(p), devaddr(ρ), devaddrs(v), devaddr(ptype32), h_))
    setfield!(p, :handle, h_[])
    finalizer(p) do x
        getfield(x, :handle) == C_NULL || ccall((:sph_destroy, libgcsph), Cvoid, (Ptr{Cvoid},), getfield(x, :handle))
        setfield!(x, :handle, C_NULL)
    end
    p
end

"""
    stepsolve!(prob::SPHProblem, n::Int = 1; timestepping = false, timelims = (sqrt(eps()), CFL H / 3c₀))

src/sphproblem.jl:204-345 -- `sph_step`; returns (updaten, maxcΔxout).  When
update! ran inside, the cell list's `cellpnum`, `pairs` and `pairsn` are
refreshed with update!'s capacity policy.
"""
function stepsolve!(prob::SPHProblem, n::Int = 1; timestepping = false,
                    timelims = (sqrt(eps()), prob.CFL * prob.H / 3prob.c₀))
    if timestepping && timelims[1] > timelims[2] error("timelims[1] should be < timelims[2]") end
    c = getfield(prob, :system)
    un, mc = Ref{Int64}(0), Ref{Cdouble}(0)
    check(ccall((:sph_step, libgcsph), Cint, (Ptr{Cvoid}, Int32, Cint, Cdouble, Cdouble, Ptr{Int64}, Ptr{Cdouble}),
                getfield(prob, :handle), n, timestepping, timelims[1], timelims[2], un, mc))
    pull_params!(prob)
    if un[] > 0
        refresh_cellpnum!(c)
        total = Ref{Int64}(0)
        check(ccall((:gcl_emit_pairs, libgcsph), Cint, (Ptr{Cvoid}, UInt64, Int64, Cint, Ptr{Int64}),
                    c.handle, UInt64(0), 0, 0, total), (GCSPH_ECAPACITY,))
        apply_update_policy!(c, Int(total[]), true)
    end
    (Int(un[]), mc[])
end

"""
    timesolve!(prob::SPHProblem; batch = 10, timeframe = 1.0, timestepping = false, timelims, verbose = true)

The compute loop of src/sphproblem.jl:420-511: stepsolve!(prob, batch)
while etime ≤ timeframe.  Frames are written by the caller between batches
(writevtk of the reference, or the Python mirror's vtkio); the animation
needs a graphics stack and is not offered.
"""
function timesolve!(prob::SPHProblem; batch = 10, timeframe = 1.0, timestepping = false,
                    timelims = (sqrt(eps()), prob.CFL * prob.H / 3prob.c₀), verbose = true)
    lim = prob.CFL * prob.H / 3prob.c₀
    if timelims[2] > lim
        @warn "Maximum dt limit ($(timelims[2])) > CFL*H/3c₀ ($lim)"
    end
    if timestepping timelims = (max(timelims[1], eps()), min(timelims[2], lim)) end
    diag = (0, 0.0)
    i = 0
    while prob.etime <= timeframe
        diag = stepsolve!(prob, batch; timestepping = timestepping, timelims = timelims)
        i += 1
    end
    verbose && println("iter: $i, time: $(prob.etime), Δt: $(prob.Δt), updn: $(diag[1]), dxpncu: $(diag[2])")
    diag
end

get_points(prob::SPHProblem) = prob.system.points      # src/sphproblem.jl:348-390
get_velocity(prob::SPHProblem) = prob.v
get_density(prob::SPHProblem) = prob.ρ
get_pressure(prob::SPHProblem) = prob.P
get_acceleration(prob::SPHProblem) = prob.∑∂v∂t
get_dpccorr(prob::SPHProblem) = prob.buf2
get_simtime(prob::SPHProblem) = prob.etime
get_dt(prob::SPHProblem) = prob.Δt
get_sumw(prob::SPHProblem) = prob.∑W
get_sumgradw(prob::SPHProblem) = prob.∑∇W
get_ptype(prob::SPHProblem) = prob.ptype

# ---------------------------------------------------------------- exported kernel functions
# src/gpukernels_sph.jl; one thread per pair with FP64 atomics in the
# library, argument order as in the reference.  `pairs` is the cell list's
# pair array (rows (0, 0) past pairsn are skipped); kernel arguments take
# the WendlandC2 kernel of the array's dimension; ptype is a CuArray{Int32},
# as the reference's examples build it (examples/animate.jl:32).

P32(pairs) = devaddr(pairs)
np(pairs) = length(pairs)

sphW!(W, pairs, points, H⁻¹, kernel) = check(ccall((:gcsph_sphW, libgcsph), Cint,
    (Int32, Int64, Int64, UInt64, Ptr{UInt64}, Cdouble, UInt64, Ptr{Cvoid}),
    length(points), length(points[1]), np(pairs), P32(pairs), devaddrs(points), H⁻¹, devaddr(W), stream()))

sph∇W!(∇W, pairs, points, H⁻¹, kernel) = check(ccall((:gcsph_sphgradW, libgcsph), Cint,
    (Int32, Int64, Int64, UInt64, Ptr{UInt64}, Cdouble, Ptr{UInt64}, Ptr{Cvoid}),
    length(points), length(points[1]), np(pairs), P32(pairs), devaddrs(points), H⁻¹, devaddrs(∇W), stream()))

sph∑W!(∑W, pairs, points, kernel, H⁻¹, ptype) = check(ccall((:gcsph_sphsumW, libgcsph), Cint,
    (Int32, Int64, Int64, UInt64, Ptr{UInt64}, Cdouble, UInt64, UInt64, Ptr{Cvoid}),
    length(points), length(points[1]), np(pairs), P32(pairs), devaddrs(points), H⁻¹, devaddr(ptype::CuArray{Int32}),
    devaddr(∑W), stream()))

sph∑∇W!(∑∇W, pairs, points, kernel, H⁻¹, ptype) = check(ccall((:gcsph_sphsumgradW, libgcsph), Cint,
    (Int32, Int64, Int64, UInt64, Ptr{UInt64}, Cdouble, UInt64, Ptr{UInt64}, Ptr{Cvoid}),
    length(points), length(points[1]), np(pairs), P32(pairs), devaddrs(points), H⁻¹,
    devaddr(ptype::CuArray{Int32}), devaddrs(∑∇W), stream()))

∂ρ∂tDDT!(∑∂ρ∂t, pairs, ∇W, ρ, v, points, h, m₀, ρ₀, c₀, γ, g, δᵩ, ptype) = check(ccall(
    (:gcsph_drhodt_ddt, libgcsph), Cint,
    (Int32, Int64, Int64, UInt64, Ptr{UInt64}, UInt64, Ptr{UInt64}, Ptr{UInt64}, Cdouble, Cdouble, Cdouble,
     Cdouble, Int32, Cdouble, Cdouble, UInt64, UInt64, Ptr{Cvoid}),
    length(points), length(points[1]), np(pairs), P32(pairs), devaddrs(∇W), devaddr(ρ), devaddrs(v),
    devaddrs(points), h, m₀, ρ₀, c₀, γ, g, δᵩ, devaddr(ptype::CuArray{Int32}), devaddr(∑∂ρ∂t), stream()))

pressure!(P, ρ, c₀, γ, ρ₀, ptype) = check(ccall((:gcsph_pressure, libgcsph), Cint,
    (Int64, UInt64, Cdouble, Int32, Cdouble, UInt64, UInt64, Ptr{Cvoid}),
    length(ρ), devaddr(ρ), c₀, γ, ρ₀, devaddr(ptype::CuArray{Int32}), devaddr(P), stream()))

∂v∂t!(∑∂v∂t, ∇W, P, pairs, m₀, ρ, ptype) = check(ccall((:gcsph_dvdt, libgcsph), Cint,
    (Int32, Int64, Int64, UInt64, Ptr{UInt64}, UInt64, Cdouble, UInt64, UInt64, Ptr{UInt64}, Ptr{Cvoid}),
    length(∑∂v∂t), length(∑∂v∂t[1]), np(pairs), P32(pairs), devaddrs(∇W), devaddr(P), m₀, devaddr(ρ),
    devaddr(ptype::CuArray{Int32}), devaddrs(∑∂v∂t), stream()))

∂v∂t_av!(∑∂v∂t, ∇W, pairs, points, h, ρ, α, v, c₀, m₀, ptype) = check(ccall((:gcsph_dvdt_av, libgcsph), Cint,
    (Int32, Int64, Int64, UInt64, Ptr{UInt64}, Ptr{UInt64}, Cdouble, UInt64, Cdouble, Ptr{UInt64}, Cdouble, Cdouble,
     UInt64, Ptr{UInt64}, Ptr{Cvoid}),
    length(points), length(points[1]), np(pairs), P32(pairs), devaddrs(∇W), devaddrs(points), h, devaddr(ρ), α,
    devaddrs(v), c₀, m₀, devaddr(ptype::CuArray{Int32}), devaddrs(∑∂v∂t), stream()))

∂v∂t_visc!(∑∂v∂t, ∇W, v, ρ, points, pairs, h, m₀, 𝜈, ptype) = check(ccall((:gcsph_dvdt_visc, libgcsph), Cint,
    (Int32, Int64, Int64, UInt64, Ptr{UInt64}, Ptr{UInt64}, UInt64, Ptr{UInt64}, Cdouble, Cdouble, Cdouble, UInt64,
     Ptr{UInt64}, Ptr{Cvoid}),
    length(points), length(points[1]), np(pairs), P32(pairs), devaddrs(∇W), devaddrs(v), devaddr(ρ),
    devaddrs(points), h, m₀, 𝜈, devaddr(ptype::CuArray{Int32}), devaddrs(∑∂v∂t), stream()))

∂v∂t_addgrav!(∑∂v∂t, gvec) = check(ccall((:gcsph_addgrav, libgcsph), Cint,
    (Int32, Int64, Cdouble, Ptr{UInt64}, Ptr{Cvoid}),
    length(∑∂v∂t), length(∑∂v∂t[1]), gvec[2], devaddrs(∑∂v∂t), stream()))   # gravvec: (0, g[, 0])

fbmolforce!(∑∂v∂t, pairs, points, d, r₀, ptype) = check(ccall((:gcsph_fbmolforce, libgcsph), Cint,
    (Int32, Int64, Int64, UInt64, Ptr{UInt64}, Cdouble, Cdouble, UInt64, Ptr{UInt64}, Ptr{Cvoid}),
    length(points), length(points[1]), np(pairs), P32(pairs), devaddrs(points), d, r₀,
    devaddr(ptype::CuArray{Int32}), devaddrs(∑∂v∂t), stream()))

∂v∂tpF!(∑∂v∂t, pairs, points, s, h, m₀, ptype) = check(ccall((:gcsph_dvdt_pF, libgcsph), Cint,
    (Int32, Int64, Int64, UInt64, Ptr{UInt64}, Cdouble, Cdouble, Cdouble, UInt64, Ptr{UInt64}, Ptr{Cvoid}),
    length(points), length(points[1]), np(pairs), P32(pairs), devaddrs(points), s, h, m₀,
    devaddr(ptype::CuArray{Int32}), devaddrs(∑∂v∂t), stream()))

dpcreg!(∑Δvdpc, v, ρ, P, pairs, points, kernel, l₀, Pmin, Pmax, Δt, λ, dpckernlim, ptype) = check(ccall(
    (:gcsph_dpcreg, libgcsph), Cint,
    (Int32, Int64, Int64, Ptr{UInt64}, Ptr{UInt64}, UInt64, UInt64, UInt64, Ptr{UInt64}, Cdouble, Cdouble, Cdouble,
     Cdouble, Cdouble, Cdouble, UInt64, Ptr{Cvoid}),
    length(points), length(points[1]), np(pairs), devaddrs(∑Δvdpc), devaddrs(v), devaddr(ρ), devaddr(P),
    P32(pairs), devaddrs(points), l₀, Pmin, Pmax, Δt, λ, dpckernlim, devaddr(ptype::CuArray{Int32}), stream()))

xsphcorr!(∑Δvxsph, pairs, W, ρ, v, m₀, 𝜀, ptype) = check(ccall((:gcsph_xsphcorr, libgcsph), Cint,
    (Int32, Int64, Int64, Ptr{UInt64}, UInt64, UInt64, UInt64, Ptr{UInt64}, Cdouble, Cdouble, UInt64, Ptr{Cvoid}),
    length(v), length(v[1]), np(pairs), devaddrs(∑Δvxsph), P32(pairs), devaddr(W), devaddr(ρ), devaddrs(v), m₀, 𝜀,
    devaddr(ptype::CuArray{Int32}), stream()))

cspmcorr!(∑ρcspm, W, ρ, m₀, pairs, ptype) = check(ccall((:gcsph_cspmcorr, libgcsph), Cint,
    (Int32, Int64, Int64, Ptr{UInt64}, UInt64, UInt64, Cdouble, UInt64, UInt64, Ptr{Cvoid}),
    length(∑ρcspm), length(ρ), np(pairs), devaddrs(∑ρcspm), devaddr(W), devaddr(ρ), m₀, P32(pairs),
    devaddr(ptype::CuArray{Int32}), stream()))

end # module
