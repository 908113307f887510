"""tk_gb300 -- GB300 (sm_103a) two-site DMRG H_eff behind tensorkraft's operator surface.

The numeric work runs in libtk_heff.so (hand-written CUDA); this package is
the host-side mirror of the reference's types and the ctypes binding.
"""
from . import _abi, symmetry
from ._abi import PREC_BF16X3, PREC_FP64, TkError
from .heff import (DavidsonSolver, EigenResult, Environment, Heff2Plan, LanczosSolver, MPO, build_heff_single_site,
                   build_heff_two_site, context)
from .symmetry import QIndex, BlockSparseTensor

__all__ = ["PREC_FP64", "PREC_BF16X3", "TkError", "Environment", "MPO", "Heff2Plan", "LanczosSolver", "DavidsonSolver",
           "EigenResult", "build_heff_two_site", "build_heff_single_site", "QIndex", "BlockSparseTensor", "context", "symmetry", "_abi"]
