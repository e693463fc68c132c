"""GB300-native scan insertion for vdb_mapping-style occupancy maps.

The compute path is libvdb_gb300.so (hand-written sm_103a CUDA behind the C
ABI in include/vdb_gb300.h); this package is its Python face, mirroring the
reference's OccupancyVDBMapping API.
"""
from .mapping import Config, Grid, MapBatch, MapServer, OccupancyVDBMapping, createIndexBoundingBox  # noqa: F401
from ._lib import VdbgError, load  # noqa: F401
