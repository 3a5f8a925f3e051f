# JumpGPU.jl -- the Julia side of the drop-in boundary: ccall bindings of
# libjumpmpm.so (include/jump_mpm.h) and methods of jump's solver entry points
#
#   solve_explicit_dynamics_2D(grid::Grid2D, solids, basis, alg::USL|MUSL, output, fixes, data)
#       SolveExplicitSolidMechanics2D.jl:24 (MUSL), :335 (USL)
#   solve_explicit_dynamics_3D(grid::Grid3D, solids, basis, alg::USL|MUSL, output, fixes, data)
#       SolveExplicitSolidMechanics3D.jl:14 (MUSL), :230 (USL)
#
# that run the time loop on one GB300, plus an ensemble call over the batched
# entry points and a ChainRulesCore.rrule over the reverse-mode entry points.
#
# A maintainer adds it to jump next to Problem.jl (`include("JumpGPU.jl")`
# after the reference modules are loaded, or `using .JumpGPU`).  The struct
# layouts below are field-for-field those of include/jump_mpm.h; the test
# tests/test_abi_layout.py parses this file and checks every struct (names,
# types, C offsets) and every ccall signature against the header, so a header
# change that is not mirrored here fails the test suite.
#
# Arrays are passed without copies: Vector{SVector{d,Float64}} and
# Vector{SMatrix{d,d,Float64}} are isbits arrays whose memory is the AoS /
# column-major layout the ABI takes, and grid.fixedNodes::Array{Int64,2} of size
# (d, nodeCount) is passed as is.  The library keeps no Julia pointer after a
# call returns.
module JumpGPU

using StaticArrays
using ChainRulesCore
using Grid, Solid, Material, Algorithm, Basis, Fix, Dirichlet, Output
import Problem

const lib = normpath(joinpath(@__DIR__, "..", "lib", "libjumpmpm.so"))
const ABI = 10  # JUMP_MPM_ABI_VERSION of the structures below

function __init__()
    v = ccall((:mpm_abi_version, lib), Cint, ())
    v == ABI || error("libjumpmpm has ABI version $v, this binding $ABI: rebuild the library")
end

# ---------------------------------------------------------------------------
# the structures of include/jump_mpm.h

struct MaterialDesc
    type::Int32
    reserved::Int32
    E::Float64
    nu::Float64
    density::Float64
    fy::Float64
    k1::Float64
    A::Float64
    B::Float64
    C::Float64
    n::Float64
    epsdot0::Float64
    cellsize::Float64
    m::Float64
    chi::Float64
    Cp::Float64
    d1::Float64
    d2::Float64
    d3::Float64
    d4::Float64
    d5::Float64
    depsdot0::Float64
    Tr::Float64
    Tm::Float64
    v_rigid::NTuple{3,Float64}
    fixed::Int32
    reserved2::Int32
end

struct GridDesc
    dim::Int32
    reserved::Int32
    xmin::NTuple{3,Float64}
    xmax::NTuple{3,Float64}
    nodes::NTuple{3,Int64}
    fixed_nodes::Ptr{Int64}
end

struct BodyDesc
    count::Int64
    mat::MaterialDesc
    pos::Ptr{Float64}
    velocity::Ptr{Float64}
    mass::Ptr{Float64}
    volume::Ptr{Float64}
    volume_initial::Ptr{Float64}
    F::Ptr{Float64}
    strain::Ptr{Float64}
    stress::Ptr{Float64}
    alpha::Ptr{Float64}
    pstrain::Ptr{Float64}
    youngs::Ptr{Float64}
    alphadot::Ptr{Float64}
    damage_init::Ptr{Float64}
    damage::Ptr{Float64}
    temperature::Ptr{Float64}
    vmstr::Ptr{Float64}
end

struct BodyView
    pos::Ptr{Float64}
    velocity::Ptr{Float64}
    volume::Ptr{Float64}
    F::Ptr{Float64}
    strain::Ptr{Float64}
    stress::Ptr{Float64}
    alpha::Ptr{Float64}
    pstrain::Ptr{Float64}
    vmstr::Ptr{Float64}
    alphadot::Ptr{Float64}
    damage_init::Ptr{Float64}
    damage::Ptr{Float64}
    temperature::Ptr{Float64}
end

struct Params
    dt::Float64
    tolerance::Float64
    body_force::NTuple{3,Float64}
    precision::Int32
    contact::Int32
    friction::Float64
    sort_interval::Int32
    flags::Int32
    algorithm::Int32
    basis::Int32
    alpha::Float64
end

struct InstanceDesc
    grid::GridDesc
    bodies::Ptr{BodyDesc}
    nbodies::Int32
    contact::Int32
    dt::Float64
    tolerance::Float64
    body_force::NTuple{3,Float64}
    friction::Float64
end

const NULL = Ptr{Float64}(0)
fptr(x) = Ptr{Float64}(pointer(x))
check(rc) = rc == 0 || error(unsafe_string(ccall((:mpm_last_error, lib), Cstring, ())))

# ---------------------------------------------------------------------------
# jump's types -> descriptors

matcode(::ElasticMaterial) = 0
matcode(::NeoHookeanMaterial) = 1
matcode(::ElastoPlasticMaterial) = 2
matcode(::JohnsonCookMaterial) = 3
matcode(::VoceMaterial) = 4
matcode(::JohnsonCookMaterialWithDamage) = 5
matcode(::RigidMaterial) = 6
# the strength part carries E, nu, the hardening constants and alpha/alphadot/vmStr
strength(m) = m isa JohnsonCookMaterialWithDamage ? m.strength_part : m
field(m, s::Symbol, default) = hasproperty(m, s) ? Float64(getproperty(m, s)) : default
fyk1(m) = m isa ElastoPlasticMaterial ? (m.fy, m.k1) : (0.0, 0.0)
hard(m::JohnsonCookMaterial) = (m.A, m.B, m.C, m.n, m.epsdot0, m.cellsize)
hard(m::VoceMaterial) = (m.A, m.B, m.C, 0.0, 0.0, m.cellsize)
hard(m::JohnsonCookMaterialWithDamage) = hard(m.strength_part)
hard(m) = (0.0, 0.0, 0.0, 0.0, 0.0, 0.0)
function dmgx(m)
    m isa JohnsonCookMaterialWithDamage || return ntuple(_ -> 0.0, 11)
    s, d = m.strength_part, m.damage_part
    (s.m, s.χ, s.Cp, d.d1, d.d2, d.d3, d.d4, d.d5, d.epsdot0, d.Tr, d.Tm)
end
# RigidMaterial as the USL solver reads it (SolveExplicitSolidMechanics2D.jl:453-461):
# vx, vy (and vz), fixed; the reference type itself holds only the density
rigidv(m) = m isa RigidMaterial ? (field(m, :vx, 0.0), field(m, :vy, 0.0), field(m, :vz, 0.0)) : (0.0, 0.0, 0.0)
rigidfixed(m) = m isa RigidMaterial && hasproperty(m, :fixed) && Bool(m.fixed) ? Int32(1) : Int32(0)
rate(m) = m isa Union{JohnsonCookMaterial,VoceMaterial,JohnsonCookMaterialWithDamage}
dmg(m) = m isa JohnsonCookMaterialWithDamage
j2(m) = m isa ElastoPlasticMaterial
basiscode(::LinearBasis) = Int32(0)
basiscode(::QuadBsplineBasis) = Int32(1)
basiscode(::CubicBsplineBasis) = Int32(2)

function material_desc(m)
    sm = strength(m)
    fy, k1 = fyk1(m)
    E = field(sm, :E, 0.0)
    nu = field(sm, :nu, 0.0)
    MaterialDesc(matcode(m), 0, E, nu, sm.density, fy, k1, hard(m)..., dmgx(m)..., rigidv(m), rigidfixed(m), 0)
end

pstrain_ptr(s, m) = j2(m) ? (length(s.pos[1]) == 2 ? fptr(m.pstrain) : fptr(m.pstrain_3D)) : NULL

function body_desc(s; youngs = NULL)
    m = s.mat
    sm = strength(m)
    BodyDesc(s.parCount, material_desc(m),
             fptr(s.pos), fptr(s.velocity), fptr(s.mass), fptr(s.volume), fptr(s.volumeInitial),
             fptr(s.deformationGradient), fptr(s.strain), fptr(s.stress),
             (j2(m) || rate(m)) ? fptr(sm.alpha) : NULL, pstrain_ptr(s, m), youngs,
             rate(m) ? fptr(sm.alphadot) : NULL,
             dmg(m) ? fptr(m.damage_init) : NULL, dmg(m) ? fptr(m.dam) : NULL,
             dmg(m) ? fptr(m.damage_part.temp) : NULL,
             hasproperty(sm, :vmStr) ? fptr(sm.vmStr) : NULL)
end

function body_view(s)
    m = s.mat
    sm = strength(m)
    BodyView(fptr(s.pos), fptr(s.velocity), fptr(s.volume), fptr(s.deformationGradient),
             fptr(s.strain), fptr(s.stress),
             (j2(m) || rate(m)) ? fptr(sm.alpha) : NULL, pstrain_ptr(s, m),
             hasproperty(sm, :vmStr) ? fptr(sm.vmStr) : NULL,
             rate(m) ? fptr(sm.alphadot) : NULL,
             dmg(m) ? fptr(m.damage_init) : NULL, dmg(m) ? fptr(m.dam) : NULL,
             dmg(m) ? fptr(m.damage_part.temp) : NULL)
end

# Grid2D/Grid3D keep lx, not xmax: xmin + lx reproduces the constructor's xmax up
# to rounding, so a caller that needs bit-exact node spacing passes xmax itself
function grid_desc(grid, dim; xmax = nothing)
    if dim == 2
        hi = xmax === nothing ? (grid.xmin + grid.lx, grid.ymin + grid.ly, 0.0) : (xmax[1], xmax[2], 0.0)
        GridDesc(2, 0, (grid.xmin, grid.ymin, 0.0), hi, (grid.nodeCountX, grid.nodeCountY, 1),
                 Ptr{Int64}(pointer(grid.fixedNodes)))
    else
        hi = xmax === nothing ? (grid.xmin + grid.lx, grid.ymin + grid.ly, grid.zmin + grid.lz) : Tuple(xmax)
        GridDesc(3, 0, (grid.xmin, grid.ymin, grid.zmin), hi, (grid.nodeCountX, grid.nodeCountY, grid.nodeCountZ),
                 Ptr{Int64}(pointer(grid.fixedNodes)))
    end
end

gravity(data, dim) = haskey(data, "bodyforce") && hasproperty(data["bodyforce"], :g) ?
    (dim == 2 ? (data["bodyforce"].g[1], data["bodyforce"].g[2], 0.0) : Tuple(data["bodyforce"].g)) : (0.0, 0.0, 0.0)

function params(alg, basis, data, dim)
    musl = alg isa MUSL
    prec = Int32(get(Dict("f64" => 0, "f32" => 1, "dw" => 2), get(data, "precision", "f64"), 0))
    Params(data["dt"], musl ? 0.0 : alg.tolerance, gravity(data, dim), prec,
           Int32(get(data, "contact", false) ? 1 : 0), Float64(get(data, "friction", 0.0)),
           Int32(get(data, "sort_interval", 0)), Int32(0), musl ? Int32(1) : Int32(0), basiscode(basis),
           musl ? alg.alpha : 1.0)
end

function create_ctx(grid, solids, alg, basis, data, dim; youngs = nothing)
    gd = grid_desc(grid, dim; xmax = get(data, "grid_xmax", nothing))
    bodies = [body_desc(s; youngs = (youngs === nothing || k > 1) ? NULL : fptr(youngs)) for (k, s) in enumerate(solids)]
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    GC.@preserve grid solids bodies youngs begin
        check(ccall((:mpm_create, lib), Cint, (Ref{GridDesc}, Ptr{BodyDesc}, Int32, Ref{Params}, Ref{Ptr{Cvoid}}),
                    gd, bodies, Int32(length(bodies)), params(alg, basis, data, dim), ctx))
    end
    return ctx[]
end

function download!(ctx, solids)
    for (s, sol) in enumerate(solids)
        GC.@preserve sol check(ccall((:mpm_download, lib), Cint, (Ptr{Cvoid}, Int32, Ref{BodyView}),
                                     ctx, Int32(s - 1), body_view(sol)))
    end
end

destroy(ctx) = ccall((:mpm_destroy, lib), Cint, (Ptr{Cvoid},), ctx)

# ---------------------------------------------------------------------------
# the solver loop

# the times of `while t < Tf ... t += dtime` (:373, :580) in FP64, one per step
function step_times(t, Tf, dt)
    ts = Float64[]
    while t < Tf
        push!(ts, t)
        t += dt
    end
    ts
end

# Steps c = 0, 1, ... run at ts[c+1]; the hooks (plotParticles_*, compute(fixes, t),
# :574-578) follow step c when c % output.interval == 0.  All steps between two
# hooks go to the library in one mpm_step call, and the particle arrays are
# downloaded into the solids only before a hook and at the end.
function gpu_solve(grid, solids, basis, alg::Union{USL,MUSL}, output, fixes, data, dim)
    ts = step_times(data["time"]::Float64, data["total_time"]::Float64, data["dt"]::Float64)
    fix_Dirichlet_grid(grid, data; ghostcell = haskey(data, "ghostcell"))
    ctx = create_ctx(grid, solids, alg, basis, data, dim)
    try
        nsteps = length(ts)
        iv = output.interval
        c = 0
        while c < nsteps
            h = c % iv == 0 ? c : c + iv - c % iv          # next hook step
            n = min(h, nsteps - 1) - c + 1
            check(ccall((:mpm_step, lib), Cint, (Ptr{Cvoid}, Int64, Ptr{Float64}), ctx, Int64(n), C_NULL))
            c += n
            if h < nsteps
                download!(ctx, solids)
                dim == 2 ? plotParticles_2D(output, solids, [grid.lx, grid.ly], [grid.nodeCountX, grid.nodeCountY], h) :
                           plotParticles_3D(output, solids, [grid.lx, grid.ly, grid.lz],
                                            [grid.nodeCountX, grid.nodeCountY, grid.nodeCountZ], h)
                compute(fixes, ts[h + 1])
            end
        end
        download!(ctx, solids)
        check(ccall((:mpm_download_grid, lib), Cint, (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                    ctx, fptr(grid.mass), fptr(grid.momentum0), fptr(grid.momentum), fptr(grid.force)))
    finally
        destroy(ctx)
    end
    closeFile(fixes)
end

# With only EnergiesFix hooks nothing reads the particle arrays between hooks:
# many hook intervals run in one call, each hook's sums formed on the device
# after its step and all of them copied back at the end (mpm_step_energies).
function gpu_energies_run!(ctx, fix::EnergiesFix, dim, n, interval, counter0, times)
    first = mod(-counter0, interval)
    nrec = n > first ? div(n - 1 - first, interval) + 1 : 0
    out = zeros(Float64, 2 + dim, max(nrec, 1))   # per record: KE, SE, momentum (dim)
    check(ccall((:mpm_step_energies, lib), Cint, (Ptr{Cvoid}, Int64, Int64, Int64, Ptr{Float64}, Ptr{Float64}),
                ctx, Int64(n), Int64(interval), Int64(first), C_NULL, out))
    for r in 1:nrec
        c = counter0 + first + (r - 1) * interval
        push!(fix.recordTime, times[c + 1]); push!(fix.kinEnergy, out[1, r]); push!(fix.strEnergy, out[2, r])
    end
end

# the drop-in: methods more specific than the reference's (grid, solids, basis, alg::USL, ...)
const GPUBasis = Union{LinearBasis,QuadBsplineBasis,CubicBsplineBasis}
Problem.solve_explicit_dynamics_2D(grid::Grid2D, solids, basis::GPUBasis, alg::Union{USL,MUSL}, output, fixes, data) =
    gpu_solve(grid, solids, basis, alg, output, fixes, data, 2)
Problem.solve_explicit_dynamics_3D(grid::Grid3D, solids, basis::GPUBasis, alg::Union{USL,MUSL}, output, fixes, data) =
    gpu_solve(grid, solids, basis, alg, output, fixes, data, 3)

# ---------------------------------------------------------------------------
# many independent problems in one batched solve (no counterpart in the
# reference, which solves one problem per call): problems[i] = (grid, solids,
# alg::USL, data) as one solve_explicit_dynamics_2D/3D call takes them; every
# problem advances nsteps steps and its solids are updated in place
function solve_ensemble!(problems, nsteps::Integer; precision = "f64")
    dim = problems[1][1] isa Grid2D ? 2 : 3
    descs = [[body_desc(s) for s in p[2]] for p in problems]
    for p in problems
        fix_Dirichlet_grid(p[1], p[4]; ghostcell = haskey(p[4], "ghostcell"))
    end
    GC.@preserve problems descs begin
        insts = [InstanceDesc(grid_desc(p[1], dim), pointer(descs[i]), Int32(length(descs[i])),
                              Int32(get(p[4], "contact", false) ? 1 : 0), p[4]["dt"], p[3].tolerance,
                              gravity(p[4], dim), Float64(get(p[4], "friction", 0.0)))
                 for (i, p) in enumerate(problems)]
        b = Ref{Ptr{Cvoid}}(C_NULL)
        check(ccall((:mpm_batch_create, lib), Cint, (Ptr{InstanceDesc}, Int32, Int32, Ref{Ptr{Cvoid}}),
                    insts, Int32(length(insts)), precision == "f32" ? Int32(1) : Int32(0), b))
        try
            check(ccall((:mpm_batch_step, lib), Cint, (Ptr{Cvoid}, Int64), b[], Int64(nsteps)))
            for (i, p) in enumerate(problems), (s, sol) in enumerate(p[2])
                check(ccall((:mpm_batch_download, lib), Cint, (Ptr{Cvoid}, Int32, Int32, Ref{BodyView}),
                            b[], Int32(i - 1), Int32(s - 1), body_view(sol)))
            end
        finally
            ccall((:mpm_batch_destroy, lib), Cint, (Ptr{Cvoid},), b[])
        end
    end
    problems
end

# ---------------------------------------------------------------------------
# differentiating through the solver: a ChainRulesCore.rrule over the reverse
# mode (the Python counterpart is jump_gb300.adjoint.Rollout, a
# torch.autograd.Function).  rollout_x(E, v0, ...) gives the final positions
# (dim per particle, all bodies in order) of an nsteps-step USL run whose single
# solid has per-particle Young's modulus E and initial velocities v0; its
# pullback runs mpm_bwd (checkpoints every `every` steps, recomputation between).

function rollout(E::Vector{Float64}, v0::Vector{Float64}, grid, solids, alg::USL, data, nsteps, every)
    dim = grid isa Grid2D ? 2 : 3
    s = solids[1]
    copyto!(reinterpret(Float64, s.velocity), v0)
    fix_Dirichlet_grid(grid, data; ghostcell = haskey(data, "ghostcell"))
    ctx = create_ctx(grid, solids, alg, LinearBasis(), data, dim; youngs = E)
    check(ccall((:mpm_fwd_checkpointed, lib), Cint, (Ptr{Cvoid}, Int64, Int32), ctx, Int64(nsteps), Int32(every)))
    download!(ctx, solids)
    return ctx, copy(reinterpret(Float64, s.pos))
end

rollout_x(args...) = (r = rollout(args...); destroy(r[1]); r[2])

function ChainRulesCore.rrule(::typeof(rollout_x), E, v0, grid, solids, alg, data, nsteps, every)
    ctx, x = rollout(E, v0, grid, solids, alg, data, nsteps, every)
    function pullback(x̄)
        Ē = similar(E)
        v̄0 = similar(v0)
        x̄c = collect(Float64, unthunk(x̄))
        try
            check(ccall((:mpm_bwd, lib), Cint,
                        (Ptr{Cvoid}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                        ctx, x̄c, C_NULL, Ē, v̄0, C_NULL))
        finally
            destroy(ctx)
        end
        return NoTangent(), Ē, v̄0, NoTangent(), NoTangent(), NoTangent(), NoTangent(), NoTangent(), NoTangent()
    end
    return x, pullback
end

end # module
