"""GB300-native (sm_103a) drop-in for scikit_tt's tensor-train ALS hot path.

Same import layout as scikit_tt: ``scikit_tt_gb300.tensor_train.TT``,
``scikit_tt_gb300.solvers.sle.als``, ``scikit_tt_gb300.solvers.evp.als``,
``scikit_tt_gb300.models.ising``.  All numerical work of the hot path runs in
``libttals.so`` (hand-written CUDA, C ABI in ``include/ttals.h``).
"""
from .tensor_train import TT  # noqa: F401
from . import solvers  # noqa: F401
