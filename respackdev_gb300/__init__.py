"""GB300-native (sm_103a) drop-in for RESPACK's cRPA polarization path (chiqw).

The compute lives in ``lib/librespack_gb300.so`` (CUDA kernels + C ABI declared
in ``include/respack_gb300.h``); :mod:`respackdev_gb300.chiqw` is the Python
mirror of that ABI, ``bin/rp_calc_chiqw`` the drop-in for the ``calc_chiqw``
executable.  Build with ``python -m respackdev_gb300.build``.
"""
from .chiqw import (PREC_BF16X3, PREC_FP16X2, PREC_FP16X3, PREC_FP64, Context, Params, calc_chiqw, default_params,  # noqa: F401
                    library_path, load, parse_namelist)
