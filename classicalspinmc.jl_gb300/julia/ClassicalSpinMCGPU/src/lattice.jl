# lattice.jl -- Lattice(shape, uc, S; bc, initialCondition) (lattice.jl:65-291 of
# ClassicalSpinMC.jl) without the per-site lookup tables: the tables are
# flattened on the library side (csmc_lattice_plan, O(N * terms)) and live on
# the device.  The fields hdf5.jl reads (S, spins, unit_cell, bc, size, shape,
# site_positions) are kept with their meaning, so the reference's file
# writers accept this Lattice.

"""The C description of a lattice and the arrays its pointers point into."""
mutable struct LatticeDesc
    arrays::Vector{Any}
    desc::Base.RefValue{CsmcLatticeDesc}
end

# row-major flattening of the C description: m[a*3+b] = M[a,b]
rowmajor(M::AbstractArray{Float64}) = vec(permutedims(M, ndims(M):-1:1))

function LatticeDesc(uc::UnitCell{D}, shape::NTuple{D,Int64}, S::Real, bc::String) where {D}
    bc in ("periodic", "open") || error("Invalid boundary condition option")
    keep = Any[]
    i32(v) = (a = Vector{Int32}(v); push!(keep, a); isempty(a) ? Ptr{Int32}(C_NULL) : pointer(a))
    f64(v) = (a = Vector{Float64}(v); push!(keep, a); isempty(a) ? Ptr{Float64}(C_NULL) : pointer(a))
    offs(o) = Int32[o...]
    field_b = [Int32(f[1]) for f in uc.field]
    field_v = reduce(vcat, [Float64.(f[2]) for f in uc.field]; init=Float64[])
    ons_b = [Int32(o[1]) for o in uc.onsite]
    ons_m = reduce(vcat, [rowmajor(ClassicalSpinMC.IMToMatrix(o[2])) for o in uc.onsite]; init=Float64[])
    bil_b = reduce(vcat, [Int32[t[1], t[2]] for t in uc.bilinear]; init=Int32[])
    bil_m = reduce(vcat, [rowmajor(ClassicalSpinMC.IMToMatrix(t[3])) for t in uc.bilinear]; init=Float64[])
    bil_o = reduce(vcat, [offs(t[4]) for t in uc.bilinear]; init=Int32[])
    cub_b = reduce(vcat, [Int32[t[1], t[2], t[3]] for t in uc.cubic]; init=Int32[])
    cub_t = reduce(vcat, [rowmajor(t[4]) for t in uc.cubic]; init=Float64[])
    cub_o = reduce(vcat, [vcat(offs(t[5]), offs(t[6])) for t in uc.cubic]; init=Int32[])
    qua_b = reduce(vcat, [Int32[t[1], t[2], t[3], t[4]] for t in uc.quartic]; init=Int32[])
    qua_t = reduce(vcat, [rowmajor(t[5]) for t in uc.quartic]; init=Float64[])
    qua_o = reduce(vcat, [vcat(offs(t[6]), offs(t[7]), offs(t[8])) for t in uc.quartic]; init=Int32[])
    sh = ntuple(k -> Int32(k <= D ? shape[k] : 1), 3)
    d = CsmcLatticeDesc(Int32(D), Int32(length(uc.basis)), sh, Int32(bc == "periodic"), Float64(S),
                        Int32(length(uc.field)), i32(field_b), f64(field_v),
                        Int32(length(uc.onsite)), i32(ons_b), f64(ons_m),
                        Int32(length(uc.bilinear)), i32(bil_b), f64(bil_m), i32(bil_o),
                        Int32(length(uc.cubic)), i32(cub_b), f64(cub_t), i32(cub_o),
                        Int32(length(uc.quartic)), i32(qua_b), f64(qua_t), i32(qua_o))
    LatticeDesc(keep, Ref(d))
end

"""
    Lattice(shape, uc, S=1/2; bc="periodic", initialCondition=:random)

The reference's Lattice constructor (lattice.jl:65-291): spins 3 x N in the
reference's site order (basis slowest), random (`:random`) or all along one
random direction (`:fm`).  The interaction tables are checked and flattened by
the library (`csmc_lattice_plan`); the lattice keeps their summary in `info`.
"""
mutable struct Lattice{D}
    S::Real
    spins::Matrix{Float64}
    unit_cell::UnitCell{D}
    bc::String
    size::Int64
    shape::NTuple{D,Int64}
    site_positions::Matrix{Float64}
    desc::LatticeDesc
    info::CsmcLatticeInfo
end

function Lattice(shape::NTuple{D,Int64}, uc::UnitCell{D}, S::Real=1 / 2; bc::String="periodic",
                 initialCondition::Symbol=:random) where {D}
    isempty(uc.basis) && addBasisSite!(uc, zeros(Float64, D))  # lattice.jl:68-70
    N = prod(shape) * length(uc.basis)
    spins = zeros(Float64, 3, N)
    if initialCondition == :random
        for i in 1:N
            set_spin!(spins, random_spin_orientation(S), i)
        end
    elseif initialCondition == :fm
        s = random_spin_orientation(S)
        for i in 1:N
            set_spin!(spins, s, i)
        end
    end
    desc = LatticeDesc(uc, shape, S, bc)
    info = CsmcLatticeInfo()
    GC.@preserve desc c_lattice_plan(desc.desc, info)
    pos = ClassicalSpinMC.compute_site_positions(uc, shape)
    Lattice{D}(S, spins, uc, bc, N, shape, pos, desc, info)
end

# deepcopy(lattice) (monte_carlo.jl:74): a new description, the same spins
function Base.deepcopy_internal(l::Lattice{D}, ::IdDict) where {D}
    c = Lattice(l.shape, deepcopy(l.unit_cell), l.S; bc=l.bc, initialCondition=:none)
    c.spins .= l.spins
    c
end

"""read_spin_configuration!(lat, filename) (hdf5.jl:266-270): lat.spins from a configuration file."""
function read_spin_configuration!(lat::Lattice, filename::String)
    h5open(filename, "r") do f
        lat.spins[:, :] = read(f["spins"])
    end
    lat
end

"""read_lattice(fid) (hdf5.jl:152-162): the lattice of a params file, built for the device."""
function read_lattice(fid)
    l = fid["lattice"]
    shape = tuple(read(l["size"])...)
    uc = ClassicalSpinMC.read_unit_cell(fid)
    Lattice(shape, uc, read(l["S"]); bc=read(l["bc"]))
end
