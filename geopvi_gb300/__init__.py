"""GB300-native engine for GeoPVI's acoustic FWI forward/adjoint path.

Drop-in modules:
  geopvi_gb300.aco2d      -- the Cython module ``aco2d`` (fwi, forward)
  geopvi_gb300.posterior  -- ``Posterior`` / ``ForwardModel`` / ``prepare_fwi_parameters``
  geopvi_gb300.fwi3d      -- the 3-D posterior (``Posterior``, ``Fwi3dEngine``, file helpers)
  geopvi_gb300.vi         -- flows, priors and the VI loop kept on the device
  geopvi_gb300.data       -- observed-data generation (``waveform.npy`` layout)
Engine:
  geopvi_gb300.engine     -- ``Fwi2dEngine``: batched device API over the C ABI
  geopvi_gb300.scheduler  -- ``FwiServer``: uneven batches and serving on one GPU
  geopvi_gb300.replicas   -- one batch per rank (multi-GPU replicas)
  geopvi_gb300.params     -- ``Params`` and the positional parameter file
  geopvi_gb300.workloads  -- seeded synthetic configurations
"""
from .params import Params, prepare_fwi_parameters, read_paramfile, write_paramfile  # noqa: F401

__version__ = "0.1.0"
