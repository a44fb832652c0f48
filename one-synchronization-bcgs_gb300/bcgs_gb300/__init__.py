"""GB300-native reorthogonalized block classical Gram-Schmidt (BCGS) QR.

``orth`` binds the C ABI of ``liborth_gb300.so`` (CUDA kernels for sm_103a);
``inputs`` makes the seeded synthetic test matrices; ``build`` compiles the
library in-tree.
"""
from . import build, inputs, orth  # noqa: F401

__all__ = ["build", "inputs", "orth"]
