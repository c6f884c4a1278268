"""GB300-native (sm_103a) 2-D DEM time step: a drop-in for TensorDEM's step.

* :class:`DEMConfig`, :class:`IceDEM` - the reference mode: FP64, same public
  surface as ``tensordem.dem`` (src/tensordem/dem.py); :class:`CalibratedIceDEM`
  adds per-bond stiffness (src/tensordem/calibrated_dem.py).
* :class:`DEM3DConfig`, :class:`IceDEM3D` - the 3-D reference mode: FP64, same
  public surface as ``tensordem.dem3d`` (src/tensordem/dem3d.py).
* :mod:`tensordem_gb300.hm2d` - the Hertz-Mindlin cell-list engine for large
  polydisperse and bonded-sheet runs.
* :mod:`tensordem_gb300.batch` - many independent Hertz-Mindlin runs in one
  batched engine; :mod:`tensordem_gb300.serve` - the request loop on top.

All compute runs in hand-written CUDA kernels of ``libtdem_sm103.so`` (built by
``python -m tensordem_gb300.build``); there is no CPU fallback.
"""

from . import dem3d, hm2d
from .calibrated import CalibratedIceDEM
from .dem import ADDITIVE_ACCOUNTING_KEYS, DEMConfig, IceDEM
from .dem3d import DEM3DConfig, IceDEM3D
from .hm2d import HM2D, HM2DConfig, granular_gas_case

__all__ = ["ADDITIVE_ACCOUNTING_KEYS", "CalibratedIceDEM", "DEM3DConfig", "DEMConfig", "IceDEM", "IceDEM3D",
           "HM2D", "HM2DConfig", "dem3d", "granular_gas_case", "hm2d"]
