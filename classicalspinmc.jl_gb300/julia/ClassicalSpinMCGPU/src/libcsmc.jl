# libcsmc.jl -- the C ABI of libcsmc.so (include/csmc.h) as Julia ccalls.
#
# One wrapper per entry point, named after it without the `csmc_` prefix and
# prefixed `c_`; each returns after checking the status (an ErrorException
# carrying csmc_last_error otherwise).  The structs mirror the C typedefs field
# for field (isbits, C layout).

"""Path of libcsmc.so: ENV["CSMC_LIB"], else the in-tree build next to this package."""
const libcsmc = get(ENV, "CSMC_LIB", normpath(joinpath(@__DIR__, "..", "..", "..", "lib", "libcsmc.so")))

const CSMC_OK = Cint(0)
const CSMC_FP64 = Int32(0)
const CSMC_FP32 = Int32(1)
const CSMC_METROPOLIS = Int32(0)
const CSMC_METROPOLIS_ADAPTIVE = Int32(1)
const CSMC_METROPOLIS_FIXED_CONE = Int32(2)
const CSMC_METROPOLIS_CONSTRAINT = Int32(3)
const CSMC_METROPOLIS_CONSTRAINT_ADAPTIVE = Int32(4)
const CSMC_PATH_AUTO = Int32(0)
const CSMC_PATH_RESIDENT = Int32(1)
const CSMC_PATH_GLOBAL = Int32(2)
const CSMC_PATH_PER_REPLICA = Int32(3)
const CSMC_ENERGY_DIFF_STATIC_MAX = 65536

# csmc_lattice_desc
struct CsmcLatticeDesc
    dim::Int32
    n_basis::Int32
    shape::NTuple{3,Int32}
    periodic::Int32
    spin_length::Float64
    n_field::Int32
    field_basis::Ptr{Int32}
    field_vec::Ptr{Float64}
    n_onsite::Int32
    onsite_basis::Ptr{Int32}
    onsite_mat::Ptr{Float64}
    n_bilinear::Int32
    bilinear_basis::Ptr{Int32}
    bilinear_mat::Ptr{Float64}
    bilinear_offset::Ptr{Int32}
    n_cubic::Int32
    cubic_basis::Ptr{Int32}
    cubic_tensor::Ptr{Float64}
    cubic_offset::Ptr{Int32}
    n_quartic::Int32
    quartic_basis::Ptr{Int32}
    quartic_tensor::Ptr{Float64}
    quartic_offset::Ptr{Int32}
end

# csmc_lattice_info
mutable struct CsmcLatticeInfo
    n_sites::Int64
    n_colours::Int32
    n_bilinear::Int32
    n_cubic::Int32
    n_quartic::Int32
    width_bilinear::Int32
    width_cubic::Int32
    width_quartic::Int32
    n_matrices::Int32
    n_cubic_tensors::Int32
    n_quartic_tensors::Int32
    padded_sites::Int64
    n_isotropic_cubic::Int32
    n_isotropic_quartic::Int32
    CsmcLatticeInfo() = new(0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0, 0)
end

# csmc_run_params
mutable struct CsmcRunParams
    sweep_start::Int64
    n_sweeps::Int64
    t_thermalization::Int64
    overrelaxation_rate::Int32
    swap_rate::Int32
    probe_rate::Int32
    kind::Int32
    path::Int32
    resident_block::Int32
    probe_energy::Ptr{Float64}
    probe_magnetization::Ptr{Float64}
    probe_capacity::Int64
    accepted::Ptr{Float64}
    exchanged::Ptr{Float64}
    n_probes_out::Int64
    CsmcRunParams() = new(0, 0, 0, 0, 0, 0, 0, 0, 0, C_NULL, C_NULL, 0, C_NULL, C_NULL, 0)
end

# csmc_constraint
struct CsmcConstraint
    site_weights::Ptr{Float64}
    g::NTuple{3,Float64}
    q::Float64
    p::Float64
    c0::Float64
    weight::Float64
end

# csmc_tune_entry
struct CsmcTuneEntry
    path::Int32
    cluster::Int32
    block::Int32
    persistent::Int32
    ms_per_window::Float64
    chosen::Int32
end

last_error() = unsafe_string(ccall((:csmc_last_error, libcsmc), Cstring, ()))
version() = unsafe_string(ccall((:csmc_version, libcsmc), Cstring, ()))

function check(rc::Cint)
    rc == CSMC_OK || error("libcsmc (status $rc): " * last_error())
    nothing
end

# ------------------------------------------------------------ tables (host only)
c_lattice_plan(desc::Ref{CsmcLatticeDesc}, info::CsmcLatticeInfo) =
    check(ccall((:csmc_lattice_plan, libcsmc), Cint, (Ref{CsmcLatticeDesc}, Ref{CsmcLatticeInfo}), desc, info))

c_lattice_tables(desc, bs, bm, cs, ct, qs, qt, field, onsite) =
    check(ccall((:csmc_lattice_tables, libcsmc), Cint,
                (Ref{CsmcLatticeDesc}, Ptr{Int64}, Ptr{Float64}, Ptr{Int64}, Ptr{Float64}, Ptr{Int64},
                 Ptr{Float64}, Ptr{Float64}, Ptr{Float64}),
                desc, bs, bm, cs, ct, qs, qt, field, onsite))

c_lattice_colouring(desc, colour_of_site, ref_of_device, colour_start) =
    check(ccall((:csmc_lattice_colouring, libcsmc), Cint, (Ref{CsmcLatticeDesc}, Ptr{Int32}, Ptr{Int64}, Ptr{Int64}),
                desc, colour_of_site, ref_of_device, colour_start))

# ------------------------------------------------------------ contexts
function c_create(desc::Ref{CsmcLatticeDesc}, precision::Integer, n_replicas::Integer, seed::Integer)
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:csmc_create, libcsmc), Cint, (Ref{CsmcLatticeDesc}, Int32, Int32, UInt64, Ref{Ptr{Cvoid}}),
                desc, precision, n_replicas, UInt64(seed), ctx))
    ctx[]
end

function c_create_batch(descs::Vector{CsmcLatticeDesc}, reps::Vector{Int32}, precision::Integer, seed::Integer)
    ctx = Ref{Ptr{Cvoid}}(C_NULL)
    check(ccall((:csmc_create_batch, libcsmc), Cint,
                (Ptr{CsmcLatticeDesc}, Int32, Ptr{Int32}, Int32, UInt64, Ref{Ptr{Cvoid}}),
                descs, length(descs), reps, precision, UInt64(seed), ctx))
    ctx[]
end

c_destroy(ctx::Ptr{Cvoid}) = check(ccall((:csmc_destroy, libcsmc), Cint, (Ptr{Cvoid},), ctx))

function c_num_slots(ctx)
    n = Ref{Int32}(0)
    check(ccall((:csmc_num_slots, libcsmc), Cint, (Ptr{Cvoid}, Ref{Int32}), ctx, n))
    Int(n[])
end

c_lattice_info_of(ctx, lattice::Integer, info::CsmcLatticeInfo) =
    check(ccall((:csmc_lattice_info_of, libcsmc), Cint, (Ptr{Cvoid}, Int32, Ref{CsmcLatticeInfo}), ctx, lattice, info))

c_set_spins(ctx, slot::Integer, spins::Matrix{Float64}) =
    check(ccall((:csmc_set_spins, libcsmc), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), ctx, slot, spins))
c_get_spins(ctx, slot::Integer, spins::Matrix{Float64}) =
    check(ccall((:csmc_get_spins, libcsmc), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), ctx, slot, spins))
c_set_spins_all(ctx, spins::Array{Float64}) =
    check(ccall((:csmc_set_spins_all, libcsmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, spins))
c_get_spins_all(ctx, spins::Array{Float64}) =
    check(ccall((:csmc_get_spins_all, libcsmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, spins))
c_random_spins(ctx, seed::Integer) =
    check(ccall((:csmc_random_spins, libcsmc), Cint, (Ptr{Cvoid}, UInt64), ctx, UInt64(seed)))

c_set_chain_ids(ctx, ids::Vector{UInt32}) =
    check(ccall((:csmc_set_chain_ids, libcsmc), Cint, (Ptr{Cvoid}, Ptr{UInt32}), ctx, ids))
c_set_temperatures(ctx, T::Vector{Float64}) =
    check(ccall((:csmc_set_temperatures, libcsmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, T))
c_set_sigma(ctx, sigma::Vector{Float64}) =
    check(ccall((:csmc_set_sigma, libcsmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, sigma))
c_get_sigma(ctx, sigma::Vector{Float64}) =
    check(ccall((:csmc_get_sigma, libcsmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, sigma))
c_set_sigma0(ctx, sigma0::Real) =
    check(ccall((:csmc_set_sigma0, libcsmc), Cint, (Ptr{Cvoid}, Float64), ctx, sigma0))
c_set_constraint(ctx, lattice::Integer, k::Ref{CsmcConstraint}) =
    check(ccall((:csmc_set_constraint, libcsmc), Cint, (Ptr{Cvoid}, Int32, Ref{CsmcConstraint}), ctx, lattice, k))
c_clear_constraint(ctx, lattice::Integer) =
    check(ccall((:csmc_set_constraint, libcsmc), Cint, (Ptr{Cvoid}, Int32, Ptr{CsmcConstraint}), ctx, lattice, C_NULL))
c_set_lambda(ctx, lambda::Vector{Float64}) =
    check(ccall((:csmc_set_lambda, libcsmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, lambda))
c_get_lambda(ctx, lambda::Vector{Float64}) =
    check(ccall((:csmc_get_lambda, libcsmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, lambda))
c_get_permutation(ctx, replica_of_slot::Vector{Int32}) =
    check(ccall((:csmc_get_permutation, libcsmc), Cint, (Ptr{Cvoid}, Ptr{Int32}), ctx, replica_of_slot))

# ------------------------------------------------------------ hot path
c_local_field(ctx, slot::Integer, H::Matrix{Float64}) =
    check(ccall((:csmc_local_field, libcsmc), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), ctx, slot, H))
c_energy_diff(ctx, slot::Integer, sites::Vector{Int64}, new_spins::Matrix{Float64}, dE::Vector{Float64}) =
    check(ccall((:csmc_energy_diff, libcsmc), Cint,
                (Ptr{Cvoid}, Int32, Int64, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}),
                ctx, slot, length(sites), sites, new_spins, dE))
c_energy_diff_static(ctx, slot::Integer, sites::Vector{Int64}, new_spins::Matrix{Float64}, dE::Vector{Float64}) =
    check(ccall((:csmc_energy_diff_static, libcsmc), Cint,
                (Ptr{Cvoid}, Int32, Int64, Ptr{Int64}, Ptr{Float64}, Ptr{Float64}),
                ctx, slot, length(sites), sites, new_spins, dE))
c_total_energy(ctx, E::Vector{Float64}) =
    check(ccall((:csmc_total_energy, libcsmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, E))
c_magnetization(ctx, M::Vector{Float64}) =
    check(ccall((:csmc_magnetization, libcsmc), Cint, (Ptr{Cvoid}, Ptr{Float64}), ctx, M))
c_metropolis_sweep(ctx, kind::Integer, accepted::Vector{Float64}) =
    check(ccall((:csmc_metropolis_sweep, libcsmc), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}), ctx, kind, accepted))
c_metropolis_sweep_at(ctx, kind::Integer, T::Vector{Float64}, accepted::Vector{Float64}) =
    check(ccall((:csmc_metropolis_sweep_at, libcsmc), Cint, (Ptr{Cvoid}, Int32, Ptr{Float64}, Int32, Ptr{Float64}),
                ctx, kind, T, length(T), accepted))
c_overrelax_sweep(ctx) = check(ccall((:csmc_overrelax_sweep, libcsmc), Cint, (Ptr{Cvoid},), ctx))
c_deterministic_sweeps(ctx, n::Integer) =
    check(ccall((:csmc_deterministic_sweeps, libcsmc), Cint, (Ptr{Cvoid}, Int64), ctx, n))
c_replay(ctx, slot::Integer, kind::Integer, T::Real, sigma::Ref{Float64}, sites::Vector{Int64},
         u_phi::Vector{Float64}, u_z::Vector{Float64}, u_acc::Vector{Float64}, accepted::Vector{UInt8}) =
    check(ccall((:csmc_replay, libcsmc), Cint,
                (Ptr{Cvoid}, Int32, Int32, Float64, Ref{Float64}, Int64, Ptr{Int64}, Ptr{Float64}, Ptr{Float64},
                 Ptr{Float64}, Ptr{UInt8}),
                ctx, slot, kind, T, sigma, length(sites), sites, u_phi, u_z, u_acc, accepted))
c_run(ctx, p::CsmcRunParams) = check(ccall((:csmc_run, libcsmc), Cint, (Ptr{Cvoid}, Ref{CsmcRunParams}), ctx, p))
c_anneal(ctx, temps::Vector{Float64}, t_therm::Integer, or_rate::Integer, kind::Integer, sigma0::Real,
         path::Integer, accepted::Union{Ptr{Nothing},Vector{Float64}}) =
    check(ccall((:csmc_anneal, libcsmc), Cint,
                (Ptr{Cvoid}, Ptr{Float64}, Int32, Int64, Int32, Int32, Float64, Int32, Ptr{Float64}),
                ctx, temps, length(temps), t_therm, or_rate, kind, sigma0, path, accepted))

# ------------------------------------------------------------ tuning and diagnostics (this library's own)
c_set_cluster_size(ctx, ranks::Integer) =
    check(ccall((:csmc_set_cluster_size, libcsmc), Cint, (Ptr{Cvoid}, Int32), ctx, ranks))
function c_cluster_size(ctx)
    r = Ref{Int32}(0)
    check(ccall((:csmc_cluster_size, libcsmc), Cint, (Ptr{Cvoid}, Ref{Int32}), ctx, r))
    Int(r[])
end
c_set_size_groups(ctx, on::Bool) = check(ccall((:csmc_set_size_groups, libcsmc), Cint, (Ptr{Cvoid}, Int32), ctx, on))
function c_size_groups(ctx)
    r = Ref{Int32}(0)
    check(ccall((:csmc_size_groups, libcsmc), Cint, (Ptr{Cvoid}, Ref{Int32}), ctx, r))
    Int(r[])
end
c_structure_factor(ctx, lattice::Integer, dim::Integer, positions::Matrix{Float64}, ks::Matrix{Float64},
                   Suv::Array{Float64,3}) =
    check(ccall((:csmc_structure_factor, libcsmc), Cint,
                (Ptr{Cvoid}, Int32, Int32, Ptr{Float64}, Int64, Ptr{Float64}, Ptr{Float64}),
                ctx, lattice, dim, positions, size(ks, 2), ks, Suv))
c_set_tensor_cores(ctx, on::Bool) = check(ccall((:csmc_set_tensor_cores, libcsmc), Cint, (Ptr{Cvoid}, Int32), ctx, on))
c_selftest_timeout(ctx, which::Integer) =
    ccall((:csmc_selftest_timeout, libcsmc), Cint, (Ptr{Cvoid}, Int32), ctx, which)
c_set_persistent(ctx, on::Bool) = check(ccall((:csmc_set_persistent, libcsmc), Cint, (Ptr{Cvoid}, Int32), ctx, on))
function c_persistent(ctx)
    r = Ref{Int32}(0)
    check(ccall((:csmc_persistent, libcsmc), Cint, (Ptr{Cvoid}, Ref{Int32}), ctx, r))
    r[] != 0
end
function c_autotune(ctx, p::CsmcRunParams, n_windows::Integer; capacity::Integer=64)
    entries = Vector{CsmcTuneEntry}(undef, capacity)
    n = Ref{Int32}(0)
    check(ccall((:csmc_autotune, libcsmc), Cint,
                (Ptr{Cvoid}, Ref{CsmcRunParams}, Int32, Ptr{CsmcTuneEntry}, Int32, Ref{Int32}),
                ctx, p, n_windows, entries, capacity, n))
    entries[1:min(Int(n[]), capacity)]
end
c_set_renormalize(ctx, every::Integer) =
    check(ccall((:csmc_set_renormalize, libcsmc), Cint, (Ptr{Cvoid}, Int32), ctx, every))
function c_spin_length_drift(ctx)
    d = Ref{Float64}(0.0)
    check(ccall((:csmc_spin_length_drift, libcsmc), Cint, (Ptr{Cvoid}, Ref{Float64}), ctx, d))
    d[]
end
function c_debug_philox(ctr::Matrix{UInt32}, key::Matrix{UInt32})
    out = similar(ctr)
    check(ccall((:csmc_debug_philox, libcsmc), Cint, (Ptr{UInt32}, Ptr{UInt32}, Int64, Ptr{UInt32}),
                ctr, key, size(ctr, 2), out))
    out
end
function c_debug_device_allocs()
    n = Ref{Int64}(0)
    check(ccall((:csmc_debug_device_allocs, libcsmc), Cint, (Ref{Int64},), n))
    n[]
end
function c_last_run_stats(ctx)
    ms, n, kms, kn = Ref{Float64}(0), Ref{Int64}(0), Ref{Float64}(0), Ref{Int64}(0)
    check(ccall((:csmc_last_run_stats, libcsmc), Cint, (Ptr{Cvoid}, Ref{Float64}, Ref{Int64}, Ref{Float64}, Ref{Int64}),
                ctx, ms, n, kms, kn))
    (device_ms=ms[], launches=n[], sweep_kernel_ms=kms[], sweep_kernel_launches=kn[])
end
