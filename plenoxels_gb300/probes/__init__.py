"""ctypes binding of libpgb_probes.so, the device-memory probes the benchmark reports
beside its roofline (random 32 B sector reads and float4 atomics). A measurement helper,
built by plenoxels_gb300.build next to the renderer and not part of its C ABI."""
from __future__ import annotations

import ctypes
import os
from ctypes import c_int32, c_int64, c_uint64, c_void_p

LIB_PATH = os.path.join(os.path.dirname(os.path.abspath(__file__)), "libpgb_probes.so")

_P = c_void_p
SIGNATURES = {
    "pgb_probe_random_reads": (c_int32, [_P, c_int64, c_int64, c_uint64, _P, _P]),
    "pgb_probe_random_atomics": (c_int32, [_P, c_int64, c_int64, c_uint64, _P]),
}
_lib = None


def load() -> ctypes.CDLL:
    """Loads the probe library once; raises RuntimeError when it has not been built."""
    global _lib
    if _lib is None:
        if not os.path.exists(LIB_PATH):
            raise RuntimeError(f"{LIB_PATH} is missing; build it with `python -m plenoxels_gb300.build`")
        lib = ctypes.CDLL(LIB_PATH)
        for name, (res, args) in SIGNATURES.items():
            fn = getattr(lib, name)
            fn.restype = res
            fn.argtypes = args
        _lib = lib
    return _lib
