"""qspectra_gb300 — GB300-native Liouville-space propagation for QSpectra models.

Drop-in for the reference's dynamical-model interface on the hot path:
Redfield (and HEOM) equations of motion, the RK4 time loop behind
simulate_dynamics / linear_response / absorption_spectra /
third_order_response, disorder ensembles and the Fourier transform, all
computed by hand-written sm_103a kernels behind the C ABI in include/qsx.h.
"""
from .bath import DebyeBath, PseudomodeBath
from .constants import CM_FS, CM_FS_LINEAR, CM_K, GAUSSIAN_SD_FWHM
from .dynamics.base import DynamicalModel, SystemOperator
from .dynamics.liouville_space import (EquationOfMotion, LiouvilleSpaceModel,
                                       LiouvilleSpaceOperator, ket_vec_to_matrix,
                                       matrix_to_bra_vec, matrix_to_ket_vec)
from .dynamics.heom import HEOMModel
from .dynamics.redfield import RedfieldModel
from .dynamics.zofe import ZOFEModel
from .hamiltonian import ElectronicHamiltonian, HamiltonianError
from .operator_tools import (SubspaceError, all_states, basis_transform_operator,
                             basis_transform_vector, n_excitations, unit_vec)
from .polarization import check_polarizations, polarization_vector
from .pulse import CustomPulse, GaussianPulse, Pulse
from .simulate.eom import simulate_dynamics, simulate_pump, simulate_with_fields
from .simulate.response import (PUMP_PROBE_PATHWAYS, THIRD_ORDER_PATHWAYS,
                                absorption_spectra, impulsive_probe,
                                linear_response, third_order_response,
                                two_dimensional_spectra)
from .simulate.utils import (IntegratorError, bound_signal, fourier_transform,
                             integrate)
from ._native import QsxError

__all__ = [
    'DebyeBath', 'PseudomodeBath', 'ZOFEModel', 'CM_FS', 'CM_FS_LINEAR', 'CM_K', 'GAUSSIAN_SD_FWHM',
    'DynamicalModel', 'SystemOperator', 'EquationOfMotion',
    'LiouvilleSpaceModel', 'LiouvilleSpaceOperator', 'ket_vec_to_matrix',
    'matrix_to_bra_vec', 'matrix_to_ket_vec', 'RedfieldModel', 'HEOMModel',
    'ElectronicHamiltonian', 'HamiltonianError', 'SubspaceError', 'all_states',
    'basis_transform_operator', 'basis_transform_vector', 'n_excitations',
    'unit_vec', 'check_polarizations', 'polarization_vector',
    'simulate_dynamics', 'simulate_with_fields', 'simulate_pump', 'Pulse', 'CustomPulse',
    'GaussianPulse', 'PUMP_PROBE_PATHWAYS', 'THIRD_ORDER_PATHWAYS',
    'absorption_spectra', 'impulsive_probe', 'linear_response',
    'third_order_response', 'two_dimensional_spectra', 'IntegratorError',
    'bound_signal', 'fourier_transform', 'integrate', 'QsxError',
]
