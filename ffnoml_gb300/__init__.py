"""ffnoml_gb300: the FFNO3D forward pass and input VJP of harshmathur1990/FFNOML on one GB300 (sm_103a).

create_ffno3d / FFNO3D are the drop-in module (reference names and call signature); the arithmetic runs in the
hand-written CUDA kernels of libffnoml_gb300.so (C ABI in include/ffnoml_gb300.h)."""
from .config import ATOM_CONFIG, MODEL_CONFIG
from .factory import create_ffno3d
from .model import FFNO3D

__all__ = ["ATOM_CONFIG", "MODEL_CONFIG", "FFNO3D", "create_ffno3d"]
