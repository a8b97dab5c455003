"""artemis_gb300 -- GB300-native (sm_103a) ray-tracing hot path for Kobra.

The product is libkgr.so (artemis_gb300/lib), built from artemis_gb300/csrc
by artemis_gb300.build: the BVH builders and refit, closest- and any-hit
traversal, the wavefront path tracer with next-event estimation, ReSTIR DI
and GI, the learned radiance cache (tcgen05 inference), tone mapping and
denoising, the batcher, autotuner and render server, and Kobra project
ingestion, behind the C ABI of include/kgr.h and include/kgr_serve.h.  This
package only binds that library (artemis_gb300.kgr).
"""
from . import kgr  # noqa: F401

__all__ = ["kgr"]
