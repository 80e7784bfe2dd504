"""GB300-native spatial-join hot path of SedonaDB (sm_103a CUDA behind the
reference's gpuspatial C ABI).

Python surface:
  capi      ctypes bindings of include/gpuspatial_c.h and include/spj_gb300.h
            (Runtime, FloatIndex2D, Refiner: the reference's wrapper surface;
            SpatialJoin, KnnJoin, StreamProbe, LearnedIndex: the extensions)
  wkb       Arrow binary WKB columns as numpy buffers
  datagen   seeded synthetic workloads
  geoparquet  GeoParquet WKB columns read onto the device; a GeoParquet writer
  materialize joined-batch gathers and the visited bitmap on the device
"""
from .wkb import WkbColumn  # noqa: F401

__all__ = ["WkbColumn"]
