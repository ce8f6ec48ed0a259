"""GB300-native panorama stitch path (sm_103a CUDA behind a C ABI).

Per camera frame: LUT gain, bilinear remap through dst->src maps into an
equirectangular canvas; then the integer multiband blend of all cameras down
to 8-bit BGR.  The kernels live in libpanostitch.so (built in-tree by
``panostitcher_gb300.build``); this package only binds and drives them.
"""
from ._lib import PsError, PhotoParam, Image, lib  # noqa: F401
from .render import (CudaPanoramaRender2, CudaTilingMultibandBlendFast, render_batch,  # noqa: F401
                     generate_reproject_map_and_mask, reproject_to_16s, get_lut, as_image)

__all__ = ["CudaPanoramaRender2", "CudaTilingMultibandBlendFast", "render_batch",
           "generate_reproject_map_and_mask", "reproject_to_16s", "get_lut", "as_image", "PsError",
           "PhotoParam", "Image", "lib"]
