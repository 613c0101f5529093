"""smallproject_gb300: GB300-native Voxel ReSTIR (sm_103a CUDA kernels behind a C ABI).

The renderer lives in libvxr.so (C++ host + CUDA); this package is its ctypes
binding plus the build script. See include/vxr.h for the C ABI.
"""
from .vxr import (World, View, SceneDesc, ViewDesc, FrameConsts, VxrError, load, check, scene_preset,  # noqa: F401
                  scene_height, camera_path, view_desc, exported_symbols, GBUF_DTYPE, RES_DTYPE, LIGHT_DTYPE,
                  LIGHTS_AREA, LIGHTS_POINT, STAGE_ALBEDO, STAGE_CANDIDATES, STAGE_SPATIAL, STAGE_SHADE,
                  STAGE_ACCUMULATE, STAGE_PATH_TRACE, LIB_PATH, Camera, PinnedBuffer, Batch, BATCH_MAX_VIEWS, BATCH_GRAPH, Tuning, tuning,
                  sky_lights, BLUE_NOISE_WORDS)
