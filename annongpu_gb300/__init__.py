"""GB300-native VMC inner loop with the pyANNonGPU interface.

    import annongpu_gb300 as pyANNonGPU

exposes PsiRBM, PsiDeep, PsiCNN, Operator, Spins, PauliString, MonteCarloSpins /
MonteCarloLoop, MonteCarloPaulis, ExactSummationSpins, ExactSummationPaulis,
ExpectationValue, TDVP, HilbertSpaceDistance and the free functions of the
reference's _pyANNonGPU module, backed by libannongpu.so (CUDA, sm_103a).
"""

from .expression import (PauliExpression, heisenberg_j1j2_2d, identity, sigma_x, sigma_y, sigma_z,  # noqa: F401
                         square_lattice_bonds, transverse_field_ising_1d, transverse_field_ising_2d)
from .json_numpy import NumpyDecoder, NumpyEncoder  # noqa: F401
from .api import (MADE, Batch, ExactSummationPaulis, ExactSummationSpins, ExpectationValue, HilbertSpaceDistance,  # noqa: F401
                  MonteCarloLoop, MonteCarloPaulis, MonteCarloSpins, Operator, PauliString,
                  PsiCNN, PsiDeep, PsiRBM, Spins, TDVP, activation_function, apply_operator, log_psi, log_psi_batch,
                  local_energies, log_psi_s, log_psi_vector, psi_O_k, psi_O_k_vector, psi_vector, setDevice, start_profiling,
                  stop_profiling)
from .api import autotune, load_tuning, save_tuning, set_tuning, tuning_table  # noqa: F401
from .api import (KullbackLeibler, PsiClassical, PsiClassicalANN_1, PsiClassicalANN_2, PsiClassicalFP_1,  # noqa: F401
                  PsiClassicalFP_2, PsiFullyPolarized)
from .builders import new_RBM, new_classical_network, new_convolutional_network, new_deep_neural_network  # noqa: F401
from ._lib import AnnError, launch_count  # noqa: F401

__version__ = "1.0.0"
