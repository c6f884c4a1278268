"""GB300-native (sm_103a) 2-D DEM time step: a drop-in for TensorDEM's step.

* :class:`DEMConfig`, :class:`IceDEM` - the reference mode: FP64, same public
  surface as ``tensordem.dem`` (src/tensordem/dem.py); :class:`CalibratedIceDEM`
  adds per-bond stiffness (src/tensordem/calibrated_dem.py).
* :mod:`tensordem_gb300.hm2d` - the Hertz-Mindlin cell-list engine for large
  polydisperse and bonded-sheet runs.
* :mod:`tensordem_gb300.batch` - many independent Hertz-Mindlin runs in one
  batched engine; :mod:`tensordem_gb300.serve` - the request loop on top.

All compute runs in hand-written CUDA kernels of ``libtdem_sm103.so`` (built by
``python -m tensordem_gb300.build``); there is no CPU fallback.
"""

from . import hm2d
from .calibrated import CalibratedIceDEM
from .dem import ADDITIVE_ACCOUNTING_KEYS, DEMConfig, IceDEM
from .hm2d import HM2D, HM2DConfig, granular_gas_case

__all__ = ["ADDITIVE_ACCOUNTING_KEYS", "CalibratedIceDEM", "DEMConfig", "IceDEM", "HM2D", "HM2DConfig",
           "granular_gas_case", "hm2d"]
