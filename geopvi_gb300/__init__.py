"""GB300-native engine for GeoPVI's 2-D acoustic FWI forward/adjoint path.

Drop-in modules:
  geopvi_gb300.aco2d      -- the Cython module ``aco2d`` (fwi, forward)
  geopvi_gb300.posterior  -- ``Posterior`` / ``ForwardModel`` / ``prepare_fwi_parameters``
Engine:
  geopvi_gb300.engine     -- ``Fwi2dEngine``: batched device API over the C ABI
  geopvi_gb300.params     -- ``Params`` and the positional parameter file
"""
from .params import Params, prepare_fwi_parameters, read_paramfile, write_paramfile  # noqa: F401

__version__ = "0.1.0"
