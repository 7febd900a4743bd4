"""bubblephysics_gb300 - GB300-native (sm_103a) bubble step of BubblePhysics behind its solver seam.

Modules:
  _native  ctypes binding of the C ABI (include/bubblephysics.h)
  spec     world specification arrays and their packing into the C records
  solver   Context / World (plain per-world path) / Batch (fused batched path)
  world    BubbleWorld / WorldTransaction / WorldFrame / advance(by:) host mirror
  server   continuous-batching step server (resident worlds, HBM budget, LRU eviction, p50/p99 latency)
  scenes   seeded synthetic worlds of the benchmark workloads
  build    in-tree nvcc build of the native library
"""
from . import _native
from .spec import WorldSpec, make_bubbles

__all__ = ["WorldSpec", "make_bubbles", "_native"]
