"""mmc_gb300: GB300-native per-photon tetrahedral tracing for Mesh-based Monte
Carlo (fangq/mmc).

The CUDA engine lives in libmmcgb.so (C ABI in include/mmcgb.h); this package
is its Python front: resident meshes and simulations (``core``), the
pmmc-compatible ``run(cfg) -> dict`` (``pmmc``), file formats (``io``), the
replay Jacobian and its autograd function (``replay``), batching/serving
(``serving``) and multi-rank sharding (``distributed``).
"""
from .core import Mesh, SimConfig, SimResult, simulate, simulate_batch  # noqa: F401

__version__ = "0.1.0"
