"""
    ClassicalSpinMCGPU

ClassicalSpinMC.jl's public API (src/ClassicalSpinMC.jl:6-35 of v1.0.0) with
the Monte Carlo hot path on a GB300 through libcsmc.so (include/csmc.h):
`Lattice`, `MonteCarlo`, the `Metropolis*()` sweep functions,
`overrelaxation!`, `simulated_annealing!`, `deterministic_updates!`,
`parallel_tempering!`, `total_energy`, `energy_density`, `get_local_field`,
`get_magnetization` and the structure-factor routines are reimplemented as
ccalls; the unit-cell builders, Bravais presets, reciprocal-space helpers and
the HDF5 writers are the reference package's own (re-exported), so model
scripts switch by replacing `using ClassicalSpinMC` with
`using ClassicalSpinMCGPU`.

The MPI ranks of a parallel-tempering job become the slots of one context:
`MonteCarlo(Ts::Vector{Float64}, lattice, params)` runs the whole ladder on
one GPU and writes `<outprefix>_<r>.h5` per temperature index r, the layout of
the MPI run.
"""
module ClassicalSpinMCGPU

using LinearAlgebra
using Printf
using Dates
using HDF5
using BinningAnalysis
using FunctionWrappers: FunctionWrapper

import ClassicalSpinMC
using ClassicalSpinMC: UnitCell, addBasisSite!, addBilinear!, addCubic!, addQuartic!, addZeemanCoupling!,
                       addOnSite!, reciprocal, get_allowed_wavevectors, get_k_path, get_k_plane, set_spin!,
                       random_spin_orientation, overwrite_keys!, write_MC_checkpoint, create_params_file,
                       Triangular, Square, Honeycomb, FCC, Pyrochlore, BreathingPyrochlore

include("libcsmc.jl")
include("lattice.jl")
include("monte_carlo.jl")

export UnitCell, addBasisSite!, addBilinear!, addCubic!, addQuartic!, addZeemanCoupling!, addOnSite!
export reciprocal, get_allowed_wavevectors, get_k_path, get_k_plane
export Lattice, set_spin!, random_spin_orientation
export get_magnetization
export overwrite_keys!, write_MC_checkpoint, create_params_file, read_lattice, read_spin_configuration!
export Metropolis, MetropolisAdaptive, MetropolisConstraint, MetropolisConstraintAdaptive, MetropolisFixedCone
export MonteCarlo, simulated_annealing!, deterministic_updates!, parallel_tempering!
export total_energy, energy_density, get_local_field
export Triangular, Square, Honeycomb, FCC, Pyrochlore, BreathingPyrochlore
export compute_equal_time_correlations, runEqualTimeStructureFactor!, compute_equal_time_structure_factor
# beyond the reference's list: the device-side constraint form and the batched correlations
export GPUConstraint, overrelaxation!, structure_factors

end
