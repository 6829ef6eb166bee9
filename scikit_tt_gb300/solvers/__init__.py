"""Drop-in replacements for ``scikit_tt.solvers.sle`` and ``scikit_tt.solvers.evp``."""
from . import sle, evp  # noqa: F401
