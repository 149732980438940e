"""p4gpu: GB300-native (sm_103a) likelihood engine for p4's hot path.

Felsenstein pruning over compressed site patterns x discrete-Gamma
categories on tree-heterogeneous models, the FP64 P = exp(Qt) decks it
consumes, and the MCMC proposal -> lnL loop, behind a C ABI
(include/p4gpu.h, libp4gpu.so) with p4's own call shapes.
"""
from .p4exceptions import P4Error
from .var import var

__all__ = ["P4Error", "var"]
