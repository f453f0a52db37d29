"""GB300-native (sm_103a) re-implementation of the vk_tessellated_clusters
per-frame tessellation pipeline: instances_classify, clusters_cull,
cluster_classify, triangle_split, triangle_tess_template_instantiate and the
BLAS list setup/insertion, as CUDA kernels behind a C ABI
(include/tc_tessellation.h, library _lib/libtc_gb300.so)."""

from . import layouts  # noqa: F401

__all__ = ["layouts"]
