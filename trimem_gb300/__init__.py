"""GB300 implementation of trimem's energy / gradient / neighbour-list /
edge-flip hot path.

``trimem_gb300.core`` is the drop-in for the reference's ``trimem.core``
(pybind11 module over the C ABI in ``include/trimem_gpu.h``);
``trimem_gb300.mc`` holds the Monte Carlo drivers.  The compute path runs only
on the GPU: without the built extension or without a CUDA device the calls
raise instead of falling back to the CPU.
"""
import os

PKG_DIR = os.path.dirname(os.path.abspath(__file__))
LIB_PATH = os.path.join(PKG_DIR, "libtrimem_gpu.so")


def load_core():
    """Import the native module, with a clear error if it was not built."""
    try:
        from . import core
    except ImportError as exc:  # pragma: no cover - exercised only when unbuilt
        raise ImportError(
            "trimem_gb300.core is not built; run `python -c \"import __graft_entry__ as g; g.build()\"`"
        ) from exc
    return core
