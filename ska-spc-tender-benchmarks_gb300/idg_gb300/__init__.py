"""GB300 Image-Domain Gridding: host side of the native library ``libidg_gb300.so``.

* ``idg_gb300.ops``       -- device-level gridder / degridder / subgrid FFT / adder / splitter
* ``idg_gb300.launcher``  -- the reference's launcher interface on host arrays
* ``idg_gb300.config``    -- YAML configuration, result table and CSV
* ``idg_gb300.datasets``  -- seeded synthetic observations and the uvw-driven plan
* ``python -m idg_gb300 <config.yaml> <out.csv>`` -- the benchmark driver
"""
from . import _lib
from ._lib import METADATA_DTYPE, SUBGRID_EXT_DTYPE, IdgError, VARIANT_BATCHED, VARIANT_PLAIN

__all__ = ["METADATA_DTYPE", "SUBGRID_EXT_DTYPE", "IdgError", "VARIANT_PLAIN", "VARIANT_BATCHED", "load"]


def load():
    """Load (building if needed) the native library."""
    return _lib.load()
