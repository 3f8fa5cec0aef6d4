"""GB300-native peridynamics engine: the hot path of XiaoMmingW/PD_Gpu1
(neighbour-family build, bond/state force loops, ADR and Verlet integration)
as hand-written sm_103a CUDA behind the C ABI in include/pd.h.

The CUDA library (libpd_gb300.so, built in-tree) is loaded on first use of
:mod:`pd_gpu1_gb300.engine`; importing this package alone does not touch the GPU.
"""
from ._abi import (FIELD, PD_MODE_DYNAMIC, PD_MODE_STATIC, PD_MODEL_BOND, PD_MODEL_STATE, PDCylinder, PDParams,
                   PDResult)

__all__ = ["FIELD", "PDParams", "PDCylinder", "PDResult", "PD_MODEL_BOND", "PD_MODEL_STATE", "PD_MODE_STATIC",
           "PD_MODE_DYNAMIC", "build"]


def build(force=False, verbose=False):
    """Compile libpd_gb300.so for sm_103a."""
    from .build import build as _build

    return _build(force=force, verbose=verbose)
