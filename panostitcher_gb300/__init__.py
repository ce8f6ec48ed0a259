"""GB300-native panorama stitch path (sm_103a CUDA behind a C ABI).

Per camera frame: LUT gain, bilinear remap through dst->src maps into an
equirectangular canvas; then the integer multiband blend of all cameras down
to 8-bit BGR.  The kernels live in libpanostitch.so (built in-tree by
``panostitcher_gb300.build``); this package only binds and drives them.
"""
from ._lib import (PsError, PhotoParam, Image, PlanarImage, lib, PS_FMT_YUV420P, PS_FMT_NV12,  # noqa: F401
                   PS_SEAMS_NEAREST_AXIS, PS_SEAMS_DISTANCE, PS_MAX_IN_FLIGHT)
from .render import (CudaPanoramaRender2, CudaRicohPanoramaRender, CudaTilingMultibandBlendFast,  # noqa: F401
                     render_batch,
                     generate_reproject_map_and_mask, reproject_to_16s, get_lut, as_image, as_planar,
                     cvt_bgr32_to_yuv, cvt_yuv_to_bgr32, non_intersecting_masks, distance_transform_l1,
                     load_photo_params)

__all__ = ["CudaPanoramaRender2", "CudaRicohPanoramaRender", "CudaTilingMultibandBlendFast", "render_batch",
           "generate_reproject_map_and_mask", "reproject_to_16s", "get_lut", "as_image", "as_planar",
           "cvt_bgr32_to_yuv", "cvt_yuv_to_bgr32", "non_intersecting_masks", "distance_transform_l1",
           "load_photo_params", "PsError", "PhotoParam", "Image", "PlanarImage", "lib", "PS_FMT_YUV420P",
           "PS_FMT_NV12", "PS_SEAMS_NEAREST_AXIS", "PS_SEAMS_DISTANCE", "PS_MAX_IN_FLIGHT"]
