"""fgrain_gb300: GB300-native photon transport and transmittance scanning for fgrain.

The compute path is libfgrain_cuda.so (CUDA kernels for sm_103a behind the C ABI in
include/fgrain_cuda.h); this package is a thin Python mirror of the reference crate's API over
that ABI, used by the tests and the benchmark.
"""
from .api import (  # noqa: F401
    DevelopmentConfig, DevelopmentReport, EmulsionConfig, ExposureConfig, GelatinOptics,
    GpuEngine, GpuError, Morphology, ScanConfig, ScanMode, VirtualEmulsionLayer,
    develop_emulsion, expose_emulsion, get_gpu_engine, reference_tree, replay_rays, replay_segments,
    scan_emulsion, scan_ray_hits, SEGMENT_DTYPE, Batch, render_tile, tile_params,
    PinnedArray, scan_signal, scan_backward, OTF_SIGMA_REFERENCE,
)
