"""artemis_gb300 -- GB300-native (sm_103a) ray-tracing hot path for Kobra.

The product is libkgr.so (artemis_gb300/lib), built from artemis_gb300/csrc
by artemis_gb300.build: BVH traversal (closest and any hit), the wavefront
path tracer with next-event estimation and ReSTIR DI, behind the C ABI of
include/kgr.h.  This package only binds that library (artemis_gb300.kgr).
"""
from . import kgr  # noqa: F401

__all__ = ["kgr"]
