"""deeds dense discrete registration on GB300 (sm_103a).

The product is libdeeds_gpu.so (C ABI: include/deeds_gpu.h) plus the
deedsBCV / applyBCV / applyBCVfloat command-line drivers built next to it.
``deedsbcv_gb300.api`` binds the C ABI for Python callers; ``phantom`` and
``nifti`` are the synthetic-data generator and the file formats.
"""
__version__ = "0.1.0"
