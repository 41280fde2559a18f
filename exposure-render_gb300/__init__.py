"""GB300-native Exposure Render transport path.

Host-side Python mirror of the reference API over libexposurerender.so (the
C ABI of include/er_capi.h).  Import with
importlib.import_module("exposure-render_gb300").
"""
from . import capi, runtime, scenes  # noqa: F401
