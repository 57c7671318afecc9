"""nlse_gb300: GB300-native split-step Fourier engine.

Drop-in for the backend="GPU" path of Quantum-Optics-LKB/NLSE v2.3.0
(NLSE/__init__.py): the same solver classes, out_field semantics, callbacks
and broadcasting, computed by hand-written sm_103a kernels in
libnlse_sm103.so (see include/nlse_gb300.h).
"""

__version__ = "2.3.0+gb300.1"

from . import callbacks
from .batch import out_fields
from .callbacks import adapt_delta_z, evaluate_delta_n, norm, sample
from .cnlse import CNLSE
from .cnlse_1d import CNLSE_1d
from .ddgpe import DDGPE
from .gpe import GPE
from .nlse import NLSE, count_steps
from .nlse_1d import NLSE_1d
from .nlse_3d import NLSE_3d

__all__ = [
    "NLSE", "NLSE_1d", "NLSE_3d", "CNLSE", "CNLSE_1d", "GPE", "DDGPE", "callbacks",
    "sample", "norm", "evaluate_delta_n", "adapt_delta_z", "count_steps", "out_fields",
]
