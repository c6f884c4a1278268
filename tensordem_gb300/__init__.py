"""GB300-native (sm_103a) 2-D DEM time step: a drop-in for TensorDEM's step.

* :class:`DEMConfig`, :class:`IceDEM` - the reference mode: FP64, same public
  surface as ``tensordem.dem`` (src/tensordem/dem.py).
* :mod:`tensordem_gb300.hm2d` - the Hertz-Mindlin cell-list engine for large
  polydisperse and bonded-sheet runs.

All compute runs in hand-written CUDA kernels of ``libtdem_sm103.so`` (built by
``python -m tensordem_gb300.build``); there is no CPU fallback.
"""

from .dem import ADDITIVE_ACCOUNTING_KEYS, DEMConfig, IceDEM

__all__ = ["ADDITIVE_ACCOUNTING_KEYS", "DEMConfig", "IceDEM"]
