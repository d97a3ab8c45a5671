"""GB300-native implementation of sif's exodus void-finder path.

- ``sif_gb300.pysif``: pysif's interface for the path (Field, Grid, ChainMesh,
  finders.exodus / exodus_raw) over sif's C API as libsif_gb300.so exports it.
- ``sif_gb300.device``: the same stages on device-resident torch tensors.
- ``sif_gb300.synth``: seeded Zel'dovich boxes and the radius ladder.
- ``sif_gb300.build``: compiles the CUDA library in-tree for sm_103a.
"""
from . import abi, synth  # noqa: F401

__all__ = ["abi", "synth", "pysif", "device", "build"]
