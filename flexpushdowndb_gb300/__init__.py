"""gfpdb: a GB300-native (sm_103a) relational hot path with FlexPushdownDB's
operator interface.

The product is ``libgfpdb.so`` (CUDA kernels + C++ operators behind the C ABI
in include/gfpdb.h). This package loads it (``_abi``), moves tables across
the Arrow C Data Interface (``tupleset``), builds expressions and plans in
the reference's vocabulary (``expression``, ``plan``), wraps the
operator-level entry points (``ops``) and generates the seeded synthetic
workloads (``workloads``).
"""

from ._abi import GfpdbError, lib  # noqa: F401

__all__ = ["GfpdbError", "lib", "build"]


def build(verbose: bool = False):
    from .build import build as _build

    return _build(verbose=verbose)
