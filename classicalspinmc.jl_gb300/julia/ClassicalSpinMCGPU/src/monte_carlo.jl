# monte_carlo.jl -- MonteCarlo and its drivers (metropolis.jl, monte_carlo.jl,
# hamiltonian.jl, observables.jl of ClassicalSpinMC.jl) on a libcsmc context.
#
# A MonteCarlo holds one device context with one replica per temperature: a
# single T is the reference's one MPI rank, a vector of T the ranks of a
# parallel-tempering ladder batched on the GPU (rank r = slot r).  The spins
# live on the device; `mc.lattice.spins` is refreshed from slot 0 after every
# driver call.  Per-slot views carry the fields the reference's hdf5.jl and
# observables.jl read (T, lattice, parameters, observables, outpath, corr,
# momentum_vectors), so its file writers and estimators run unchanged.

const SimulationParameters = ClassicalSpinMC.SimulationParameters
const MCParamsBuffer = ClassicalSpinMC.MCParamsBuffer
const Observables = ClassicalSpinMC.Observables

"""
    MonteCarlo(T, lattice, parameters; constraint, weight, outpath, outprefix,
               inparams, overwrite, sigma0, corr, ks, precision, seed, path)

monte_carlo.jl:56-118 on the device.  `T` is a Float64 (one replica, the
reference's signature) or a Vector{Float64} (one replica per temperature:
the MPI ranks of parallel_tempering!).  Extra keywords: `precision`
(:fp64 or :fp32), `seed` (Philox key of every random draw), `path`
(:auto, :resident, :global, :per_replica).  `constraint` is a
`GPUConstraint` (the closed form c = g.V + q|V|^2 + p|V| + c0 of
V = sum_i w_i s_i) or `nothing`.
"""
mutable struct MonteCarlo
    T::Float64
    temperatures::Vector{Float64}
    parameters::SimulationParameters
    lattice::Lattice
    observables::Vector{Observables}
    lambda::Float64
    weight::Float64
    constraint::Any
    outpath::String
    outpaths::Vector{String}
    sigma::Float64
    sigma0::Float64
    corr::Bool
    momentum_vectors::Matrix{Float64}
    ctx::Ptr{Cvoid}
    path::Int32
    accepted::Vector{Float64}
    exchanged::Vector{Float64}
end

"""The closed-form constraint the device evaluates (csmc_constraint)."""
struct GPUConstraint
    site_weights::Union{Nothing,Vector{Float64}}
    g::NTuple{3,Float64}
    q::Float64
    p::Float64
    c0::Float64
end
GPUConstraint(; site_weights=nothing, g=(0.0, 0.0, 0.0), q=0.0, p=0.0, c0=0.0) =
    GPUConstraint(site_weights, Tuple(Float64.(g)), Float64(q), Float64(p), Float64(c0))
function (k::GPUConstraint)(lat)
    w = k.site_weights === nothing ? ones(lat.size) : k.site_weights
    V = lat.spins * w
    vv = dot(V, V)
    dot(collect(k.g), V) + k.q * vv + k.p * sqrt(vv) + k.c0
end

const _PATHS = Dict(:auto => CSMC_PATH_AUTO, :resident => CSMC_PATH_RESIDENT, :global => CSMC_PATH_GLOBAL,
                    :per_replica => CSMC_PATH_PER_REPLICA)

MonteCarlo(T::Float64, lattice::Lattice{D}, parameters::Dict{String,Int64}; kw...) where {D} =
    MonteCarlo([T], lattice, parameters; kw...)

function MonteCarlo(Ts::Vector{Float64}, lattice::Lattice{D}, parameters::Dict{String,Int64};
                    constraint=nothing, weight::Float64=0.0, outpath::String="", outprefix::String="configuration",
                    inparams::Dict{String,<:Any}=Dict{String,Any}(), overwrite::Bool=true, sigma0::Real=60,
                    corr::Bool=false, ks::Matrix{Float64}=Matrix{Float64}(undef, D, 0),
                    precision::Symbol=:fp64, seed::Integer=20261203, path::Symbol=:auto) where {D}
    if corr && size(ks, 2) == 0
        error("No momentum vectors provided for correlation calculations!")
    elseif !corr && size(ks, 2) != 0
        @warn "Momentum vectors provided but correlation calculations not requested!"
    end
    constraint === nothing || constraint isa GPUConstraint ||
        error("the device evaluates a GPUConstraint (c = g.V + q|V|^2 + p|V| + c0), not an arbitrary function")
    R = length(Ts)
    R >= 1 || error("at least one temperature")
    lat = deepcopy(lattice)  # monte_carlo.jl:74
    prec = precision == :fp32 ? CSMC_FP32 : precision == :fp64 ? CSMC_FP64 : error("precision is :fp64 or :fp32")
    ctx = GC.@preserve lat c_create(lat.desc.desc, prec, R, seed)
    mc = MonteCarlo(Ts[1], copy(Ts), MCParamsBuffer(copy(parameters)), lat,
                    [Observables(size(ks, 2)) for _ in 1:R], 0.0, weight, constraint, "", String[],
                    Float64(sigma0), Float64(sigma0), corr, ks, ctx, _PATHS[path], zeros(R), zeros(R))
    finalizer(m -> m.ctx == C_NULL || (c_destroy(m.ctx); m.ctx = C_NULL), mc)
    c_set_temperatures(ctx, mc.temperatures)
    c_set_sigma(ctx, fill(Float64(sigma0), R))
    c_set_sigma0(ctx, sigma0)
    if constraint !== nothing
        w = constraint.site_weights
        k = Ref(CsmcConstraint(w === nothing ? Ptr{Float64}(C_NULL) : pointer(w), constraint.g, constraint.q,
                               constraint.p, constraint.c0, weight))
        GC.@preserve w c_set_constraint(ctx, 0, k)
    end
    for r in 0:R-1
        c_set_spins(ctx, r, lat.spins)
    end
    if length(outpath) > 0  # monte_carlo.jl:95-113, rank r -> slot r
        isdir(outpath) || mkdir(outpath)
        paramsfile = string(outpath, outprefix, ".h5.params")
        mc.outpaths = [string(outpath, outprefix, "_", r, ".h5") for r in 0:R-1]
        if !isfile(paramsfile) && overwrite
            ClassicalSpinMC.create_params_file(mc, paramsfile)
            length(inparams) > 0 && ClassicalSpinMC.write_attributes(paramsfile, inparams)
        end
        for r in 0:R-1
            if !isfile(mc.outpaths[r+1]) && overwrite
                println("Creating new file $(basename(mc.outpaths[r+1])) for output on rank $r")
                ClassicalSpinMC.initialize_hdf5(slot_view(mc, r), paramsfile)
            end
        end
        mc.outpath = mc.outpaths[1]
    end
    mc
end

nslots(mc::MonteCarlo) = length(mc.temperatures)

"""mc.lattice.spins <- slot 0 on the device."""
sync!(mc::MonteCarlo) = (c_get_spins(mc.ctx, 0, mc.lattice.spins); mc)

function slot_spins(mc::MonteCarlo, r::Integer)
    s = zeros(Float64, 3, mc.lattice.size)
    c_get_spins(mc.ctx, r, s)
    s
end

"""The fields of one rank's MonteCarlo that hdf5.jl and observables.jl read."""
struct SlotView{L}
    T::Float64
    lattice::L
    parameters::SimulationParameters
    observables::Observables
    outpath::String
    corr::Bool
    momentum_vectors::Matrix{Float64}
end

function slot_view(mc::MonteCarlo, r::Integer; spins=nothing)
    lat = mc.lattice
    view_lat = (S=lat.S, spins=spins === nothing ? slot_spins(mc, r) : spins, unit_cell=lat.unit_cell, bc=lat.bc,
                size=lat.size, shape=lat.shape, site_positions=lat.site_positions)
    out = isempty(mc.outpaths) ? "" : mc.outpaths[r+1]
    SlotView(mc.temperatures[r+1], view_lat, mc.parameters, mc.observables[r+1], out, mc.corr, mc.momentum_vectors)
end

# ------------------------------------------------------------------ sweeps
"""The body of Metropolis() etc.: one device sweep of every slot at temperature T."""
struct DeviceSweep
    kind::Int32
end
function (s::DeviceSweep)(mc::MonteCarlo, T::Float64)::Float64
    acc = zeros(nslots(mc))
    c_metropolis_sweep_at(mc.ctx, s.kind, [T], acc)
    sync!(mc)
    acc[1]
end

const SweepFn = FunctionWrapper{Float64,Tuple{MonteCarlo,Float64}}

"""Metropolis() (metropolis.jl:181-183): metropolis! (:65-82) as a device sweep."""
Metropolis()::SweepFn = SweepFn(DeviceSweep(CSMC_METROPOLIS))
"""MetropolisAdaptive() (metropolis.jl:185-187): metropolis_adaptive! (:113-133)."""
MetropolisAdaptive()::SweepFn = SweepFn(DeviceSweep(CSMC_METROPOLIS_ADAPTIVE))
"""MetropolisFixedCone() (metropolis.jl:189-191): metropolis_fixed_cone! (:136-153)."""
MetropolisFixedCone()::SweepFn = SweepFn(DeviceSweep(CSMC_METROPOLIS_FIXED_CONE))
"""MetropolisConstraint() (metropolis.jl:193-195): metropolis_constraint! (:36-58)."""
MetropolisConstraint()::SweepFn = SweepFn(DeviceSweep(CSMC_METROPOLIS_CONSTRAINT))
"""MetropolisConstraintAdaptive() (metropolis.jl:197-199): metropolis_constraint_adaptive! (:155-179)."""
MetropolisConstraintAdaptive()::SweepFn = SweepFn(DeviceSweep(CSMC_METROPOLIS_CONSTRAINT_ADAPTIVE))

# the device kind behind a sweep function, or nothing for a caller's own function
sweep_kind(alg::SweepFn) = alg.obj[] isa DeviceSweep ? alg.obj[].kind : nothing

"""overrelaxation!(mc) (monte_carlo.jl:126-139): one sweep of every slot, colour class by colour class."""
overrelaxation!(mc::MonteCarlo) = (c_overrelax_sweep(mc.ctx); sync!(mc))

# ------------------------------------------------------------------ observables
"""total_energy (hamiltonian.jl:70-132) of slot 0 (or of `slot`)."""
function total_energy(mc::MonteCarlo; slot::Integer=0)
    E = zeros(nslots(mc))
    c_total_energy(mc.ctx, E)
    E[slot+1]
end
"""energy_density (hamiltonian.jl:134-136)."""
energy_density(mc::MonteCarlo; slot::Integer=0) = total_energy(mc; slot=slot) / mc.lattice.size
"""get_magnetization (observables.jl:12-18): |sum_i s_i| of slot 0 (or of `slot`)."""
function get_magnetization(mc::MonteCarlo; slot::Integer=0)
    M = zeros(nslots(mc))
    c_magnetization(mc.ctx, M)
    M[slot+1]
end
"""get_local_field (hamiltonian.jl:3-67) at 1-based site `point`."""
function get_local_field(mc::MonteCarlo, point::Int64; slot::Integer=0)
    H = zeros(Float64, 3, mc.lattice.size)
    c_local_field(mc.ctx, slot, H)
    (H[1, point], H[2, point], H[3, point])
end

# a bare Lattice goes through a one-replica FP64 context of its own
function with_context(f, lat::Lattice)
    ctx = GC.@preserve lat c_create(lat.desc.desc, CSMC_FP64, 1, 0)
    try
        c_set_spins(ctx, 0, lat.spins)
        f(ctx)
    finally
        c_destroy(ctx)
    end
end
total_energy(lat::Lattice) = with_context(ctx -> (E = zeros(1); c_total_energy(ctx, E); E[1]), lat)
energy_density(lat::Lattice) = total_energy(lat) / lat.size
get_magnetization(lat::Lattice) = with_context(ctx -> (M = zeros(1); c_magnetization(ctx, M); M[1]), lat)
get_local_field(lat::Lattice, point::Int64) =
    with_context(ctx -> (H = zeros(3, lat.size); c_local_field(ctx, 0, H); (H[1, point], H[2, point], H[3, point])),
                 lat)
function overrelaxation!(lat::Lattice)
    with_context(lat) do ctx
        c_overrelax_sweep(ctx)
        c_get_spins(ctx, 0, lat.spins)
    end
    lat
end

# ------------------------------------------------------------------ drivers
"""
    simulated_annealing!(mc, schedule, T0=1.0; alg=Metropolis())

monte_carlo.jl:157-190: for T = T0, schedule(1), schedule(2), ... while T > mc.T,
sigma reset to sigma0 and t_thermalization-1 iterations of [overrelaxation,
alg(mc, T) every overrelaxation_rate-th], then a checkpoint.  Every slot anneals
through the same temperatures.  A device sweep kind runs as one csmc_anneal
call per temperature; a caller's own `alg` is called as the reference does.
"""
function simulated_annealing!(mc::MonteCarlo, schedule::Function, T0::Float64=1.0; alg::SweepFn=Metropolis())
    p = mc.parameters
    accept_total = p.t_thermalization * mc.lattice.size
    p.overrelaxation_rate != 0 && (accept_total /= p.overrelaxation_rate)
    kind = sweep_kind(alg)
    T, time = T0, 1
    while T > mc.T
        if kind !== nothing
            acc = zeros(nslots(mc))
            c_anneal(mc.ctx, [T], p.t_thermalization, p.overrelaxation_rate, kind, mc.sigma0, mc.path, acc)
            R = acc[1]
        else  # the reference's loop around the caller's function
            R, t = 0.0, 1
            c_set_sigma(mc.ctx, fill(mc.sigma0, nslots(mc)))
            while t < p.t_thermalization
                if p.overrelaxation_rate != 0
                    c_overrelax_sweep(mc.ctx)
                    t % p.overrelaxation_rate == 0 && (R += alg(mc, T))
                else
                    R += alg(mc, T)
                end
                t += 1
            end
        end
        println("Acceptance rate at T=$T: $(round(R / accept_total * 100, digits=5)) % ")
        T = schedule(time)
        time += 1
        sync!(mc)
        isempty(mc.outpaths) || write_checkpoints(mc)
    end
    mc
end

"""
    deterministic_updates!(mc)

monte_carlo.jl:201-213: the reference makes t_deterministic-1 single-site
alignments s_i <- -S H_i/|H_i| at random sites; here ceil((t_deterministic-1)/N)
colour sweeps visit every site once per sweep.
"""
function deterministic_updates!(mc::MonteCarlo)
    n = max(mc.parameters.t_deterministic - 1, 0)
    c_deterministic_sweeps(mc.ctx, cld(n, mc.lattice.size))
    sync!(mc)
end

function write_checkpoints(mc::MonteCarlo)
    for r in 0:nslots(mc)-1
        ClassicalSpinMC.write_MC_checkpoint(slot_view(mc, r))
    end
end
"""write_MC_checkpoint(mc) (hdf5.jl:176-181): every slot's file gets its current spins."""
ClassicalSpinMC.write_MC_checkpoint(mc::MonteCarlo) = write_checkpoints(mc)

"""
    parallel_tempering!(mc, saveIC=Int64[]; alg=Metropolis())

monte_carlo.jl:235-398 with the ranks as the slots of one context: each
report_interval is one or more csmc_run calls (cut after the sweeps whose end
state the host reads: checkpoints and IC files of the measurement phase,
correlation probes), the probe records of E and |M| are pushed into each
slot's ErrorPropagators, and at the end every slot's file receives its final
observables (write_final_observables).
"""
function parallel_tempering!(mc::MonteCarlo, saveIC::Vector{Int64}=Int64[]; alg::SweepFn=Metropolis())
    p = mc.parameters
    kind = sweep_kind(alg)
    kind === nothing && error("parallel_tempering! runs the device sweep kinds (Metropolis() ... )")
    R = nslots(mc)
    R == 1 && @warn "MPI commSize of 1; no replica exchanges will occur!"
    out = !isempty(mc.outpaths)
    total = p.t_thermalization + p.t_measurement
    for r in saveIC
        0 <= r < R || error("saveIC ranks must be in 0:$(R - 1)")
        out && (d = joinpath(dirname(mc.outpaths[r+1]), "IC_$r"); isdir(d) || mkdir(d))
    end
    is_corr(it) = mc.corr && p.probe_rate > 0 && it >= p.t_thermalization && it % p.probe_rate == 0
    is_ic(it) = (out || !isempty(saveIC)) && it >= p.t_thermalization && it % p.checkpoint_rate == 0
    @printf("Running sweeps on %s.\n", Dates.format(Dates.now(), "dd u yyyy HH:MM:SS"))
    start = 0
    while start < total
        n = min(p.report_interval, total - start)
        acc, exc = zeros(R), zeros(R)
        q = start
        for it in start:start+n-1
            (is_corr(it) || is_ic(it) || it == start + n - 1) || continue
            run_piece!(mc, q, it + 1 - q, kind, acc, exc)
            q = it + 1
            if is_corr(it)
                Suv = structure_factors(mc, mc.momentum_vectors)
                for r in 1:R
                    ClassicalSpinMC.update_correlations!(slot_view(mc, r - 1; spins=mc.lattice.spins), Suv[:, :, r])
                end
            end
            if is_ic(it)
                timestep = (it - p.t_thermalization) ÷ p.checkpoint_rate
                out && write_checkpoints(mc)
                for r in saveIC
                    out && ClassicalSpinMC.write_initial_configuration(
                        joinpath(dirname(mc.outpaths[r+1]), "IC_$r", "IC_$timestep.h5"), slot_view(mc, r))
                end
            end
        end
        mc.accepted .+= acc
        mc.exchanged .+= exc
        start += n
        print_statistics(mc, start, acc, exc, n)
    end
    sync!(mc)
    if out
        @printf("Writing observables on %s.\n", Dates.format(Dates.now(), "dd u yyyy HH:MM:SS"))
        for r in 0:R-1
            ClassicalSpinMC.write_final_observables(slot_view(mc, r))
        end
    end
    @printf("Simulation finished on %s.\n", Dates.format(Dates.now(), "dd u yyyy HH:MM:SS"))
    mc
end

# one csmc_run call over sweeps [start, start + n): its probe records go into
# the slots' ErrorPropagators (update_observables!, observables.jl:20-25)
function run_piece!(mc::MonteCarlo, start::Integer, n::Integer, kind::Int32, acc::Vector{Float64},
                    exc::Vector{Float64})
    p = mc.parameters
    R = nslots(mc)
    cap = p.probe_rate > 0 ? n ÷ p.probe_rate + 1 : 0
    E = zeros(R, max(cap, 1))  # [slot, probe]: the C side writes [probe][slot]
    M = zeros(R, max(cap, 1))
    rp = CsmcRunParams()
    rp.sweep_start, rp.n_sweeps, rp.t_thermalization = start, n, p.t_thermalization
    rp.overrelaxation_rate, rp.swap_rate, rp.probe_rate = p.overrelaxation_rate, p.swap_rate, p.probe_rate
    rp.kind, rp.path = kind, mc.path
    GC.@preserve E M acc exc begin
        rp.probe_energy, rp.probe_magnetization, rp.probe_capacity = pointer(E), pointer(M), cap
        rp.accepted, rp.exchanged = pointer(acc), pointer(exc)
        c_run(mc.ctx, rp)
    end
    for k in 1:rp.n_probes_out, r in 1:R
        ClassicalSpinMC.update_observables!(slot_view(mc, r - 1; spins=mc.lattice.spins), E[r, k], M[r, k])
    end
    sync!(mc)
end

# print_runtime_statistics! (helper.jl:25-78) for the slots of the context
function print_statistics(mc::MonteCarlo, t, acc, exc, n)
    p = mc.parameters
    total = p.t_thermalization + p.t_measurement
    sigma = zeros(nslots(mc))
    c_get_sigma(mc.ctx, sigma)
    str = @sprintf("Sweep %d / %d (%.1f%%)\n", t, total, 100.0 * t / total)
    str *= @sprintf("\t\tthermalized : %s\n", t >= p.t_thermalization ? "YES" : "NO")
    attempted = n * mc.lattice.size / max(p.overrelaxation_rate, 1)
    for r in 1:nslots(mc)
        swaps = p.swap_rate > 0 ? n / p.swap_rate / ((r == 1 || r == nslots(mc)) ? 2.0 : 1.0) : 0.0
        str *= @sprintf("\t\tsimulation %d update acceptance rate : %.2f%%\tsigma : %.2f\n", r - 1,
                        100 * acc[r] / attempted, sigma[r])
        str *= @sprintf("\t\tsimulation %d replica exchange acceptance rate : %.2f%%\n", r - 1,
                        swaps > 0 ? 100 * exc[r] / swaps : 0.0)
    end
    print(str * "\n")
end

# ------------------------------------------------------------------ correlations
"""compute_equal_time_correlations of every slot: [9, N_k, slots] (spin_correlations.jl:6-43)."""
function structure_factors(mc::MonteCarlo, ks::Matrix{Float64})
    D = size(ks, 1)
    out = zeros(Float64, 9, size(ks, 2), nslots(mc))  # C layout [slot][k][9]
    c_structure_factor(mc.ctx, 0, D, mc.lattice.site_positions, ks, out)
    out
end

"""compute_equal_time_correlations(lat or mc, ks) (spin_correlations.jl:6-43): 9 x N_k."""
compute_equal_time_correlations(mc::MonteCarlo, ks::Array{Float64,2}) = structure_factors(mc, ks)[:, :, 1]
function compute_equal_time_correlations(lat::Lattice, ks::Array{Float64,2})
    with_context(lat) do ctx
        out = zeros(Float64, 9, size(ks, 2), 1)
        c_structure_factor(ctx, 0, size(ks, 1), lat.site_positions, ks, out)
        out[:, :, 1]
    end
end

"""
    runEqualTimeStructureFactor!(path, lat, ks, override=false)

spin_correlations.jl:48-108 for one process: the IC files of every
`IC_<rank>` directory under `path` are loaded as the slots of one context, up
to 64 at a time, and their correlations computed in one device launch; each
file receives `spin_correlations/{SSF, SSF_momentum}` unless it has them and
`override` is false.
"""
function runEqualTimeStructureFactor!(path, lat::Lattice, ks::Matrix{Float64}, override=false)
    files = String[]
    for d in readdir(path; join=true)
        isdir(d) && startswith(basename(d), "IC_") || continue
        append!(files, filter(f -> endswith(f, ".h5"), readdir(d; join=true)))
    end
    todo = override ? files : filter(f -> !h5open(g -> haskey(g, "spin_correlations"), f, "r"), files)
    for chunk in Iterators.partition(todo, 64)
        ctx = GC.@preserve lat c_create(lat.desc.desc, CSMC_FP64, length(chunk), 0)
        try
            for (r, f) in enumerate(chunk)
                s = h5open(g -> read(g["spins"]), f, "r")
                c_set_spins(ctx, r - 1, s)
            end
            out = zeros(Float64, 9, size(ks, 2), length(chunk))
            c_structure_factor(ctx, 0, size(ks, 1), lat.site_positions, ks, out)
            for (r, f) in enumerate(chunk)
                h5open(f, "r+") do g
                    d = haskey(g, "spin_correlations") ? g["spin_correlations"] : create_group(g, "spin_correlations")
                    overwrite_keys!(d, Dict("SSF" => out[:, :, r], "SSF_momentum" => ks))
                end
            end
        finally
            c_destroy(ctx)
        end
    end
end

"""compute_equal_time_structure_factor(path, dest) (spin_correlations.jl:116-145): file averaging, unchanged."""
compute_equal_time_structure_factor(path::String, dest::String) =
    ClassicalSpinMC.compute_equal_time_structure_factor(path, dest)
