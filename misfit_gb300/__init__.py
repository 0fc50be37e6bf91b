"""misfit_gb300 -- GB300 implementation of MISFIT's dynamic MIS-maintenance path.

The product is the C-ABI library ``lib/libmisfit_gb.so`` (include/misfit_gb.h)
and the drop-in ``bin/misfit`` / ``bin/misfit_async`` binaries; this package
holds their sources (``csrc/``), the build recipe (``build.py``), a ctypes
binding (``native.py``) and the synthetic-workload generators
(``workloads.py``).
"""
__all__ = ["workloads", "native", "build"]
