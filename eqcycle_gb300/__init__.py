"""eqcycle_gb300 -- the eqcycle time-stepping hot path on GB300 (sm_103a).

Host side in Python mirrors the reference's Julia interface: ``set_parameters`` is
par.jl:setParameters, ``main`` is src/main.jl:main, ``Solver`` exposes the per-operator
entry points of the C ABI (include/eqc.h) implemented by libeqc.so.
"""
from .config import ModelConfig, preset, reference_config, ensemble_members, shard_members, YR2SEC  # noqa: F401
from .params import set_parameters, structured_parameters, Params  # noqa: F401
from .solver import Solver, Ensemble, main, Results  # noqa: F401
from ._lib import (EQC_FP64, EQC_MIXED, EQC_PC_AMG, EQC_PC_JACOBI, EQC_GUESS_PREVIOUS,  # noqa: F401
                   EQC_GUESS_LEARNED, EQC_GUESS_EXTRAPOLATE, EQC_TOL_RHS, EQC_TOL_R0, EqcError)
