"""GB300 implementation of RBMonGPU's variational hot path.

The public names mirror the reference's Python module (pyRBMonGPU): ``Psi``,
``PsiDeep``, ``PsiPair``, ``Operator``, ``MonteCarloLoop``, ``ExactSummation``,
``ExpectationValue``, ``HilbertSpaceDistance``, ``psi_O_k_vector``,
``activation_function``, ``setDevice`` and the network factories.  All compute
runs in the CUDA library ``librbmg.so`` (include/rbmg.h) through ctypes.
"""
from . import gradient_descent, operators
from .api import (Batch, Chain, ExactSummation, ExpectationValue, FixedSamples, HilbertSpaceDistance, MonteCarloLoop, Operator, Psi, PsiDeep,
                  PsiPair, Proposal, RbmgError, Spins, activation_function, new_deep_neural_network, new_neural_network,
                  psi_O_k_vector, get_S_matrix, DiagDensityOp, KullbackLeibler, local_energies, setDevice, start_profiling, stop_profiling, library_stream)
from .gradient_descent import Optimizer

__all__ = ["Batch", "Chain", "Proposal", "library_stream", "Psi", "PsiDeep", "PsiPair", "Operator", "Spins", "MonteCarloLoop", "ExactSummation", "FixedSamples",
           "ExpectationValue", "HilbertSpaceDistance", "psi_O_k_vector", "get_S_matrix", "DiagDensityOp", "KullbackLeibler", "local_energies", "activation_function", "setDevice",
           "start_profiling", "stop_profiling", "new_neural_network", "new_deep_neural_network", "RbmgError",
           "operators", "gradient_descent", "Optimizer"]
