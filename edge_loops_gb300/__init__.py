"""GB300-native (sm_103a) load-balanced CSR SpMV/SpMM: the `loops` schedules
(thread_mapped, group_mapped, work_oriented, merge_path) behind the C ABI of
include/edge_loops.h.  `api` is the Python face of that ABI; `synth` makes
the synthetic benchmark matrices."""
from . import _lib  # noqa: F401

__all__ = ["api", "synth", "build"]
