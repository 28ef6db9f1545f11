"""ctypes mirror of include/or3.h and the loader for libor3.so.

The loader never falls back to anything: if the CUDA library is missing or was
built for another ABI version, it raises.
"""
import ctypes
import os

from . import build as _build

c_double3 = ctypes.c_double * 3

OR3_OK = 0
OR3_ERR_INVALID_ARGUMENT = -1
OR3_ERR_CUDA = -2
OR3_ERR_OUT_OF_MEMORY = -3
OR3_ERR_NO_DEVICE = -4
OR3_ERR_NOT_FOUND = -5
OR3_ERR_DEVICE_REPORTED = -6
OR3_ERR_BUSY = -7

OR3_LAMBERT, OR3_SPECULAR, OR3_REFRACTION, OR3_PHONG = 0, 1, 2, 3
OR3_SPHERE_LIGHT = 1
OR3_PLANE_AXIS_ALIGNED, OR3_PLANE_INFINITE_FLOOR = 0, 1
OR3_LAYOUT_REFERENCE, OR3_LAYOUT_COMPACT = 0, 1
OR3_BUILD_AUTO, OR3_BUILD_HOST, OR3_BUILD_DEVICE = 0, 1, 2
OR3_BUILD_DEVICE_MIN_PRIMS = 16384
OR3_FLAG_KEEP_PATHS = 1
OR3_FLAG_NO_GRAPH = 4
OR3_FLAG_TIME_KERNELS = 16
OR3_FLAG_COUNT_TRAVERSAL = 32
OR3_FLAG_ONE_LANE = 64
OR3_FLAG_QUANTISED_NODES = 128
OR3_FLAG_HOIST_NODES = 256
OR3_FLAG_UNSORTED_SHADE = 512
OR3_FLAG_HOST_LOOP = 1024

API_VERSION = 1
OR3_API_VERSION = API_VERSION


class Material(ctypes.Structure):
    _fields_ = [("type", ctypes.c_int32), ("texture", ctypes.c_int32), ("emission", c_double3),
                ("color", c_double3), ("ior", ctypes.c_double), ("phong_exponent", ctypes.c_double)]


P = ctypes.POINTER
u32p = P(ctypes.c_uint32)
f64p = P(ctypes.c_double)
f32p = P(ctypes.c_float)


class SceneDescC(ctypes.Structure):
    _fields_ = [
        ("num_materials", ctypes.c_uint32), ("materials", P(Material)),
        ("num_layers", ctypes.c_uint32), ("layer_material", u32p), ("layer_rate", f64p),
        ("num_triangles", ctypes.c_uint32), ("tri_vertices", f64p), ("tri_normals", f64p), ("tri_uvs", f64p),
        ("tri_layers", u32p), ("tri_ids", u32p),
        ("num_spheres", ctypes.c_uint32), ("spheres", f64p), ("sphere_layers", u32p), ("sphere_flags", u32p),
        ("sphere_ids", u32p),
        ("num_planes", ctypes.c_uint32), ("planes", f64p), ("plane_layers", u32p), ("plane_ids", u32p),
        ("env_width", ctypes.c_uint32), ("env_height", ctypes.c_uint32), ("env_rgb", f32p),
        ("env_rgbe", P(ctypes.c_uint8)),
        ("background", c_double3),
        ("num_textures", ctypes.c_uint32), ("texture_dims", u32p), ("texture_offsets", P(ctypes.c_uint64)),
        ("texture_rgb", f32p), ("build", ctypes.c_uint32), ("leaf_max", ctypes.c_uint32),
        ("traversal_cost", ctypes.c_double),
    ]


class CameraC(ctypes.Structure):
    _fields_ = [("width", ctypes.c_uint32), ("height", ctypes.c_uint32), ("position", c_double3),
                ("direction", c_double3), ("up", c_double3), ("screen_height_world", ctypes.c_double),
                ("distance_to_screen", ctypes.c_double), ("focal_distance", ctypes.c_double),
                ("aperture_radius", ctypes.c_double)]


class RenderParamsC(ctypes.Structure):
    _fields_ = [("min_samples", ctypes.c_int32), ("max_samples", ctypes.c_int32),
                ("step_samples", ctypes.c_int32), ("supersamples", ctypes.c_int32),
                ("next_event_estimation", ctypes.c_int32), ("rr_min_depth", ctypes.c_int32),
                ("max_depth", ctypes.c_int32), ("output_layout", ctypes.c_int32),
                ("seed", ctypes.c_uint64), ("wave_paths", ctypes.c_uint64),
                ("flags", ctypes.c_uint32), ("tuning", ctypes.c_uint32)]


class RenderStatsC(ctypes.Structure):
    _fields_ = [("camera_paths", ctypes.c_uint64), ("extension_rays", ctypes.c_uint64),
                ("shadow_rays", ctypes.c_uint64), ("bounces", ctypes.c_uint64), ("waves", ctypes.c_uint64),
                ("render_ms", ctypes.c_double), ("upload_ms", ctypes.c_double),
                ("samples", ctypes.c_int32), ("passes", ctypes.c_int32),
                ("extend_ms", ctypes.c_double), ("shade_ms", ctypes.c_double),
                ("extend_launches", ctypes.c_uint64), ("shade_launches", ctypes.c_uint64),
                ("nodes_visited", ctypes.c_uint64), ("tris_tested", ctypes.c_uint64),
                ("spheres_tested", ctypes.c_uint64), ("shadow_ms", ctypes.c_double),
                ("shadow_launches", ctypes.c_uint64), ("lanes", ctypes.c_uint32), ("waves_rerun", ctypes.c_uint32),
                ("kernel_launches", ctypes.c_uint64)]


class SceneInfoC(ctypes.Structure):
    _fields_ = [("num_primitives", ctypes.c_uint64), ("num_nodes", ctypes.c_uint64),
                ("device_bytes", ctypes.c_uint64), ("build_ms", ctypes.c_double), ("upload_ms", ctypes.c_double),
                ("tree_depth", ctypes.c_int32), ("num_lights", ctypes.c_int32), ("flatten_ms", ctypes.c_double)]


FRAME_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_int32, f64p, ctypes.c_size_t, ctypes.c_size_t,
                            ctypes.c_double)


class BatchJobC(ctypes.Structure):
    _fields_ = [("scene", ctypes.c_int32), ("reserved", ctypes.c_uint32), ("camera", CameraC),
                ("params", RenderParamsC), ("frame_host", f64p), ("frame_capacity", ctypes.c_size_t)]


class BatchParamsC(ctypes.Structure):
    _fields_ = [("wave_paths", ctypes.c_uint64), ("flags", ctypes.c_uint32), ("graph_bounces", ctypes.c_uint32),
                ("blocks_per_sm", ctypes.c_uint32), ("reserved", ctypes.c_uint32)]


class ServerParamsC(ctypes.Structure):
    _fields_ = [("wave_paths", ctypes.c_uint64), ("hbm_budget_bytes", ctypes.c_uint64),
                ("max_active_jobs", ctypes.c_uint32), ("frame_every_samples", ctypes.c_uint32),
                ("graph_bounces", ctypes.c_uint32), ("flags", ctypes.c_uint32)]


class JobStatusC(ctypes.Structure):
    _fields_ = [("state", ctypes.c_int32), ("samples_done", ctypes.c_int32), ("submit_s", ctypes.c_double),
                ("admit_s", ctypes.c_double), ("first_frame_s", ctypes.c_double), ("done_s", ctypes.c_double)]


class ServerStatsC(ctypes.Structure):
    _fields_ = [("jobs_submitted", ctypes.c_uint64), ("jobs_done", ctypes.c_uint64),
                ("jobs_cancelled", ctypes.c_uint64), ("camera_paths", ctypes.c_uint64), ("waves", ctypes.c_uint64),
                ("busy_s", ctypes.c_double), ("device_ms", ctypes.c_double), ("latency_p50_s", ctypes.c_double),
                ("latency_p99_s", ctypes.c_double), ("queue_p50_s", ctypes.c_double),
                ("queue_p99_s", ctypes.c_double), ("first_frame_p50_s", ctypes.c_double),
                ("peak_active_jobs", ctypes.c_uint64), ("peak_budget_bytes", ctypes.c_uint64),
                ("waves_rerun", ctypes.c_uint64)]


class MeshC(ctypes.Structure):
    _fields_ = [("num_triangles", ctypes.c_uint32), ("vertices", f64p), ("normals", f64p), ("uvs", f64p),
                ("material", u32p), ("num_materials", ctypes.c_uint32), ("materials", P(Material)),
                ("material_names", P(ctypes.c_char_p)), ("texture_paths", P(ctypes.c_char_p))]


class SceneFileC(ctypes.Structure):
    _fields_ = [("desc", SceneDescC), ("num_meshes", ctypes.c_uint32), ("space_partitioning", ctypes.c_char * 16),
                ("texture_paths", P(ctypes.c_char_p)), ("ibl_path", ctypes.c_char_p)]


JOB_FRAME8_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, P(ctypes.c_uint8),
                                 ctypes.c_size_t, ctypes.c_size_t, ctypes.c_int32)
JOB_FRAME_CB = ctypes.CFUNCTYPE(None, ctypes.c_void_p, ctypes.c_uint64, ctypes.c_int32, f64p, ctypes.c_size_t,
                                ctypes.c_size_t, ctypes.c_int32)

OR3_JOB_QUEUED, OR3_JOB_RUNNING, OR3_JOB_DONE, OR3_JOB_CANCELLED, OR3_JOB_FAILED = 0, 1, 2, 3, 4
OR3_SERVER_KEEP_MOMENTS = 1
OR3_SERVER_ONE_LANE = 2
OR3_SERVER_UNSORTED_SHADE = 4
OR3_TUNE_EXTEND_MASK = 0x7
OR3_TUNE_SMEM_NODES = 0x10
OR3_TUNE_SHADOW_UNSORTED = 0x20
OR3_TUNE_L2_PERSIST = 0x40
OR3_TUNE_SHADE_NEE_OCC4 = 0x80
OR3_TUNE_ONE_LANE = 0x100
OR3_TUNE_TWO_LANES = 0x200
OR3_TUNE_FOUR_LANES = 0x400
OR3_TUNE_SORTED_SHADE = 0x800
OR3_TUNE_BLOCK_APPEND = 0x1000
OR3_TUNE_UNSORTED_SHADE = 0x2000
OR3_TUNE_WIDE8 = 0x4000
OR3_TUNE_SHADOW_REFILL8 = 0x8000

# name -> (restype, argtypes); every function declared in include/or3.h
PROTOTYPES = {
    "or3_api_version": (ctypes.c_int, []),
    "or3_context_create": (ctypes.c_int, [ctypes.c_int, P(ctypes.c_void_p)]),
    "or3_context_destroy": (ctypes.c_int, [ctypes.c_void_p]),
    "or3_last_error": (ctypes.c_char_p, [ctypes.c_void_p]),
    "or3_scene_upload": (ctypes.c_int, [ctypes.c_void_p, P(SceneDescC), P(ctypes.c_int32)]),
    "or3_scene_release": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32]),
    "or3_scene_get_info": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, P(SceneInfoC)]),
    "or3_render": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, P(CameraC), P(RenderParamsC), FRAME_CB,
                                  ctypes.c_void_p]),
    "or3_stop": (ctypes.c_int, [ctypes.c_void_p]),
    "or3_reset_stop": (ctypes.c_int, [ctypes.c_void_p]),
    "or3_get_frame": (ctypes.c_int, [ctypes.c_void_p, f64p, ctypes.c_size_t, P(ctypes.c_int32)]),
    "or3_get_stats": (ctypes.c_int, [ctypes.c_void_p, P(RenderStatsC)]),
    "or3_get_moments": (ctypes.c_int, [ctypes.c_void_p, f64p, f64p, ctypes.c_size_t, P(ctypes.c_uint64)]),
    "or3_get_path_radiance": (ctypes.c_int, [ctypes.c_void_p, f32p, ctypes.c_size_t, P(ctypes.c_uint64)]),
    "or3_trace_closest": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_size_t, f32p, f32p,
                                         P(ctypes.c_int32), f32p, f32p]),
    "or3_trace_closest_device": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_size_t, ctypes.c_void_p,
                                                ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p, ctypes.c_void_p,
                                                ctypes.c_void_p]),
    "or3_env_sample": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_size_t, f32p, f32p]),
    "or3_texture_sample": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_int32, ctypes.c_size_t, f32p,
                                          f32p]),
    "or3_trace_occluded": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, ctypes.c_size_t, f32p, f32p, f32p,
                                          P(ctypes.c_uint8)]),
    "or3_render_paths_noalloc": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, P(CameraC), P(RenderParamsC),
                                                ctypes.c_uint64, ctypes.c_uint32, ctypes.c_void_p,
                                                ctypes.c_void_p]),
    "or3_render_batch": (ctypes.c_int, [ctypes.c_void_p, P(BatchJobC), ctypes.c_size_t, P(BatchParamsC),
                                        P(RenderStatsC)]),
    "or3_get_batch_moments": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_size_t, f64p, f64p, ctypes.c_size_t,
                                             P(ctypes.c_uint64)]),
    "or3_autotune_batch": (ctypes.c_int, [ctypes.c_void_p, P(BatchJobC), ctypes.c_size_t, ctypes.c_uint64,
                                          P(BatchParamsC), P(ctypes.c_double)]),
    "or3_server_start": (ctypes.c_int, [ctypes.c_void_p, P(ServerParamsC), JOB_FRAME_CB, ctypes.c_void_p]),
    "or3_server_start8": (ctypes.c_int, [ctypes.c_void_p, P(ServerParamsC), JOB_FRAME8_CB, ctypes.c_void_p]),
    "or3_encode_rgb8": (ctypes.c_int, [ctypes.c_void_p, f64p, ctypes.c_size_t, ctypes.c_int32, P(ctypes.c_uint8)]),
    "or3_encode_rgbe": (ctypes.c_int, [ctypes.c_void_p, f64p, ctypes.c_size_t, P(ctypes.c_uint8)]),
    "or3_decode_rgbe": (ctypes.c_int, [ctypes.c_void_p, P(ctypes.c_uint8), ctypes.c_size_t, f32p]),
    "or3_get_frame_rgb8": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_int32, P(ctypes.c_uint8), ctypes.c_size_t,
                                          P(ctypes.c_int32)]),
    "or3_get_frame_rgbe": (ctypes.c_int, [ctypes.c_void_p, P(ctypes.c_uint8), ctypes.c_size_t, P(ctypes.c_int32)]),
    "or3_mesh_load_obj": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_int32, ctypes.c_uint32, P(P(MeshC))]),
    "or3_mesh_transform": (ctypes.c_int, [P(MeshC), P(ctypes.c_double), P(ctypes.c_double), P(ctypes.c_double)]),
    "or3_mesh_free": (None, [P(MeshC)]),
    "or3_read_hdr": (ctypes.c_int, [P(ctypes.c_uint8), ctypes.c_size_t, P(ctypes.c_uint32), P(ctypes.c_uint32),
                                    P(ctypes.c_uint8), ctypes.c_size_t]),
    "or3_scene_load_file": (ctypes.c_int, [ctypes.c_char_p, ctypes.c_uint32, P(P(SceneFileC)), ctypes.c_char_p,
                                           ctypes.c_size_t]),
    "or3_scene_file_free": (None, [P(SceneFileC)]),
    "or3_server_submit": (ctypes.c_int, [ctypes.c_void_p, P(BatchJobC), P(ctypes.c_uint64)]),
    "or3_server_poll": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, P(JobStatusC)]),
    "or3_server_cancel": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64]),
    "or3_server_drain": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_double]),
    "or3_server_get_stats": (ctypes.c_int, [ctypes.c_void_p, P(ServerStatsC)]),
    "or3_server_get_moments": (ctypes.c_int, [ctypes.c_void_p, ctypes.c_uint64, f64p, f64p, ctypes.c_size_t,
                                              P(ctypes.c_uint64)]),
    "or3_server_stop": (ctypes.c_int, [ctypes.c_void_p]),
}

OR3_NOALLOC_MAX_PATHS = 4096

_LIB = None


def load_library(build_if_missing=True):
    """Loads the in-tree libor3.so (building it first if asked and needed)."""
    global _LIB
    if _LIB is not None:
        return _LIB
    path = _build.LIB_PATH
    if build_if_missing and _build.needs_build():
        _build.build_library()
    if not os.path.exists(path):
        raise RuntimeError("libor3.so is not built (%s); run __graft_entry__.build()" % path)
    lib = ctypes.CDLL(path)
    for name, (res, args) in PROTOTYPES.items():
        fn = getattr(lib, name)
        fn.restype = res
        fn.argtypes = args
    if lib.or3_api_version() != API_VERSION:
        raise RuntimeError("libor3.so ABI version %d != %d" % (lib.or3_api_version(), API_VERSION))
    _LIB = lib
    return lib
