"""gbdbscan: GB300-native exact DBSCAN (drop-in for the CUDA-DClust+ pipeline).

The package directory holds the CUDA sources (csrc/), their build recipe
(build.py), the ctypes host mirror of the C ABI (api.py) and the synthetic
workload generators (datasets.py).  Import it by directory name, e.g.
``importlib.import_module("fast-cuda-gpu-dbscan_gb300")``.
"""
from .api import (GD_PREC_FP32_BAND, GD_PREC_FP64, NOISE, Context, GdError, Server,
                  import_dataset, label_quality, load_library, write_labels)

__all__ = ["Context", "Server", "GdError", "GD_PREC_FP64", "GD_PREC_FP32_BAND", "NOISE",
           "import_dataset", "label_quality", "load_library", "write_labels"]
