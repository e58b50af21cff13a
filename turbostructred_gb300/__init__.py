"""GB300-native explicit finite-volume residual and stage update (TurboStructred hot path).

The compute path is the in-tree CUDA library libtsfvm.so (include/ts_fvm.h);
:mod:`turbostructred_gb300.capi` binds it, :mod:`turbostructred_gb300.build` builds it.
"""
