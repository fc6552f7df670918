"""GB300-native Monte Carlo sweeps for ClassicalSpinMC.jl models.

Host-side mirror of the reference's public API (ClassicalSpinMC.jl,
src/ClassicalSpinMC.jl:6-35) over the C ABI of libcsmc.so: unit cells and
lattices are described on the host, flattened and coloured natively, and all
sweeps, energies, magnetisations and replica exchanges run as sm_103a CUDA
kernels.  Julia's ``!`` suffix is dropped from names.

The package directory name contains a dot, so import it through
``load()`` in ``__graft_entry__`` or by path (importlib).
"""
from ._lib import CSMCError, lib  # noqa: F401
from .lattice import Lattice, get_spin, random_spin_orientation, set_spin  # noqa: F401
from .monte_carlo import (MCParamsBuffer, Metropolis, MetropolisAdaptive, MetropolisFixedCone,  # noqa: F401
                          MetropolisConstraint, MetropolisConstraintAdaptive, Constraint, MonteCarlo, SimulationParameters, annealing_temperatures, deterministic_updates,
                          energy_density, get_local_field, get_magnetization, local_fields, overrelaxation,
                          parallel_tempering, replay, simulated_annealing, total_energy, autotune,
                          compute_equal_time_correlations, structure_factors)
from . import examples  # noqa: F401
from .observables import specific_heat, susceptibility  # noqa: F401
from .hdf5 import (create_params_file, h5open, overwrite_keys, read_lattice, read_spin_configuration,  # noqa: F401
                   write_MC_checkpoint)
from .reciprocal import get_allowed_wavevectors, get_k_path, get_k_plane, reciprocal  # noqa: F401
from .spin_correlations import compute_equal_time_structure_factor, runEqualTimeStructureFactor  # noqa: F401
from .unit_cell import (FCC, BreathingPyrochlore, Honeycomb, Pyrochlore, Square, Triangular,  # noqa: F401
                        UnitCell, addBasisSite, addBilinear, addCubic, addOnSite, addQuartic, addZeemanCoupling)
