"""GB300-native wavefront path tracer for omochi-renderer3's render call.

The compute path is libor3.so (hand-written CUDA for sm_103a behind the C ABI
in include/or3.h); this package only builds it, loads it and mirrors the
reference's render interface on top of it.
"""
from . import abi, build, renderer, scene, workloads  # noqa: F401
from .renderer import Context, GpuPathTracer, Or3Error, ScreenPixels, load_obj, load_scene_file, read_hdr  # noqa: F401
from .scene import Camera, SceneDesc  # noqa: F401
