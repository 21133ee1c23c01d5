"""dmftpack_gb300 -- GB300-native (sm_103a CUDA) DMFT self-consistency hot path of DMFTpack.

The compute lives in libdmftgpu.so (C ABI: include/dmftgpu.h); this package builds it in-tree
(:mod:`dmftpack_gb300.build`), binds it (:mod:`dmftpack_gb300.lib`) and provides the host-side helpers
for inputs: the Hk.HWR format (:mod:`dmftpack_gb300.hwr`) and the seeded synthetic workloads
(:mod:`dmftpack_gb300.models`).
"""
from .lib import Context, Lattice, DmftGpuError, kmesh  # noqa: F401
