"""FrameLab-GB300: GB300-native CT reconstruction hot path (sm_103a).

The compute lives in ``libframelab_gb300.so`` (hand-written CUDA behind a
C ABI, ``include/framelab_gb300.h``). This package is the host-side mirror of
the reference's MATLAB classes (``+Operators``, ``+DataTypes``,
``+Transforms``, ``+Optimizers``) over that ABI.
"""
__all__ = ["geometry", "phantoms"]
