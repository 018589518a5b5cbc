"""tmr_gb300 — GB300-native octree-forest adaptation path of TMR.

``tmr_gb300.TMR`` mirrors the octree part of ``tmr.TMR`` (OctForest,
Octant, OctantArray, VecInterp, MatrixFilter); ``tmr_gb300.autograd``
exposes the filter -> interpolation chain as a torch.autograd.Function.
All compute runs in the sm_103a library built by ``tmr_gb300.build``.
"""
from . import TMR  # noqa: F401

__all__ = ["TMR"]
