"""GB300-native backend for the BraketSimulator.jl ``braket_sv_v2`` / ``braket_dm_v2``
simulate path.

The numerical work runs in hand-written sm_103a CUDA kernels behind the C ABI of
``libbraket_gb300.so`` (include/braket_gb300.h); this package is the host layer
that mirrors the reference's Julia API (simulators, gates, noise, observables,
result types) and lowers each instruction onto that ABI.
"""
from . import _abi, gates, noises, observables
from .gates import *  # noqa: F401,F403  (gate types, as the reference exports them)
from .noises import (AmplitudeDamping, BitFlip, Depolarizing, GeneralizedAmplitudeDamping, Kraus,  # noqa: F401
                     MultiQubitPauliChannel, PauliChannel, PhaseDamping, PhaseFlip, TwoQubitDephasing,
                     TwoQubitDepolarizing, TwoQubitPauliChannel)
from .simulators import (DensityMatrixSimulator, Instruction, StateVectorSimulator, apply_observables,  # noqa: F401
                         density_matrix, evolve, expectation, probabilities, qubit_count, reinit, samples,
                         state_vector, state_with_observables)
from .results import (Amplitude, DensityMatrix, Expectation, Probability, Sample, StateVector, Variance,  # noqa: F401
                      calculate, marginal_probability, partial_trace, permute_density_matrix, permute_probability)
from .adjoint import adjoint_gradient, energy_rrule, parameter_shift_gradient, torch_energy  # noqa: F401
from .program import (Circuit, Program, basis_rotation_gates, create_sim, fix_endianness, simulate,  # noqa: F401
                      tensor_product_index_dict)
from .batch import CapturedBatch, batch_simulate  # noqa: F401
from .autotune import autotune, get_tuning, set_tuning  # noqa: F401


def library_path() -> str:
    return _abi.LIB_PATH


def version() -> str:
    return _abi.lib().bs_version().decode()
