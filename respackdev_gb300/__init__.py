"""GB300-native (sm_103a) drop-in for RESPACK's cRPA polarization path (chiqw)
and the Wannier-basis interaction integrals that consume it (calc_int).

The compute lives in ``lib/librespack_gb300.so`` (CUDA kernels + C ABI declared
in ``include/respack_gb300.h``); :mod:`respackdev_gb300.chiqw` and
:mod:`respackdev_gb300.calc_int` are the Python mirrors of that ABI;
``bin/rp_calc_chiqw``, ``bin/rp_calc_w3d`` and ``bin/rp_calc_j3d`` are the
drop-ins for the reference's executables.  Build with
``python -m respackdev_gb300.build``.
"""
from .chiqw import (PREC_BF16X3, PREC_FP16X2, PREC_FP16X3, PREC_FP64, Context, Params, calc_chiqw, default_params,  # noqa: F401
                    library_path, load, parse_namelist)
from . import calc_int  # noqa: F401,E402
