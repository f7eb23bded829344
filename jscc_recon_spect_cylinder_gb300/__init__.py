"""GB300-native (sm_103a) OSEM hot path for SC / JSCC SPECT on a polar grid.

Drop-in modules mirroring the reference's module names and signatures:

=====================================  =============================================
reference module                        this package
=====================================  =============================================
recon_osem_plane                        .recon_osem_plane
recon_osem_plane_sparse                 .recon_osem_plane_sparse
recon_osem_local_cntstat                .recon_osem_local_cntstat
recon_osem_local_sparse_jsccsd_only     .recon_osem_local_sparse_jsccsd_only
process_list_plane_strict               .process_list_plane_strict
process_list_plane                      .process_list_plane
process_list_plane_sparse               .process_list_plane_sparse
compton_sparse_ops                      .compton_sparse_ops
=====================================  =============================================

All compute runs in ``lib/libjscc_gb300.so`` (C-ABI in include/jscc_gb300.h). Importing
the package does not initialise CUDA, so it is safe to import in spawned workers.
"""
from __future__ import annotations

import importlib
import sys

__version__ = "0.1.0"

_MIRRORED = (
    "recon_osem_plane",
    "recon_osem_plane_sparse",
    "recon_osem_local_cntstat",
    "recon_osem_local_sparse_jsccsd_only",
    "process_list_plane_strict",
    "process_list_plane",
    "process_list_plane_sparse",
    "compton_sparse_ops",
)


def install(modules=_MIRRORED) -> None:
    """Register the mirrored modules under the reference's top-level names, so the
    reference's entry points (``from recon_osem_plane import run_recon_osem``) bind to
    this package. Call before importing the entry point."""
    for name in modules:
        sys.modules[name] = importlib.import_module(f"{__name__}.{name}")
