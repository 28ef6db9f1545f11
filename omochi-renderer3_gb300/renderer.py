"""Python host mirror of the reference's render interface over the C ABI.

`GpuPathTracer` has the reference PathTracer's constructor arguments and
methods (src/renderer/PathTracer.h:18-88, src/renderer/Renderer.h:10-23):
RenderScene, GetResult, GetCurrentSampleCount, GetCurrentRenderingInfo,
StopRendering, EnableNextEventEstimation, SetMaxThreadCount.  `Context` is a
thin owner of an or3_context; every call goes to libor3.so (CUDA) and errors
surface as `Or3Error` with the library's message.
"""
import ctypes
import threading

import numpy as np

from . import abi


class Or3Error(RuntimeError):
    def __init__(self, code, msg):
        super().__init__("or3 error %d: %s" % (code, msg))
        self.code = code


class Context:
    def __init__(self, device=0):
        self.lib = abi.load_library()
        h = ctypes.c_void_p()
        rc = self.lib.or3_context_create(device, ctypes.byref(h))
        if rc != abi.OR3_OK:
            raise Or3Error(rc, "cannot create a context on CUDA device %d" % device)
        self.h = h
        self._keep = {}

    def _check(self, rc):
        if rc != abi.OR3_OK:
            raise Or3Error(rc, self.lib.or3_last_error(self.h).decode())
        return rc

    def close(self):
        if self.h:
            self.lib.or3_context_destroy(self.h)
            self.h = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    # ---- scenes
    def upload(self, scene_desc):
        d, keep = scene_desc.to_c()
        sid = ctypes.c_int32()
        self._check(self.lib.or3_scene_upload(self.h, ctypes.byref(d), ctypes.byref(sid)))
        return sid.value

    def upload_file(self, path, threads=0, build=0):
        """A scene file straight from or3_scene_load_file to or3_scene_upload (no Python copy)."""
        lib, fp = _scene_file_open(path, threads)
        try:
            fp.contents.desc.build = build
            sid = ctypes.c_int32()
            self._check(self.lib.or3_scene_upload(self.h, ctypes.byref(fp.contents.desc), ctypes.byref(sid)))
        finally:
            lib.or3_scene_file_free(fp)
        return sid.value

    def release(self, scene):
        self._check(self.lib.or3_scene_release(self.h, scene))

    def scene_info(self, scene):
        info = abi.SceneInfoC()
        self._check(self.lib.or3_scene_get_info(self.h, scene, ctypes.byref(info)))
        return {k: getattr(info, k) for k, _ in abi.SceneInfoC._fields_}

    # ---- render
    @staticmethod
    def _params(supersamples=1, min_samples=1, max_samples=1, step_samples=1, next_event_estimation=False,
                rr_min_depth=5, max_depth=0, layout=abi.OR3_LAYOUT_REFERENCE, seed=0, wave_paths=0, flags=0,
                tuning=0):
        p = abi.RenderParamsC()
        p.min_samples, p.max_samples, p.step_samples = min_samples, max_samples, step_samples
        p.supersamples = supersamples
        p.next_event_estimation = 1 if next_event_estimation else 0
        p.rr_min_depth, p.max_depth = rr_min_depth, max_depth
        p.output_layout = layout
        p.seed, p.wave_paths, p.flags, p.tuning = seed, wave_paths, flags, tuning
        return p

    def render_paths_noalloc(self, scene, camera, first_path, num_paths, radiance_dev_ptr, stream=None,
                             **settings):
        """or3_render_paths_noalloc: radiance of paths [first, first+num) into a caller-owned device buffer."""
        cam = camera.to_c()
        p = self._params(**settings)
        self._check(self.lib.or3_render_paths_noalloc(self.h, scene, ctypes.byref(cam), ctypes.byref(p),
                                                      first_path, num_paths, ctypes.c_void_p(radiance_dev_ptr),
                                                      ctypes.c_void_p(stream)))

    def render(self, scene, camera, *, supersamples=1, min_samples=1, max_samples=1, step_samples=1,
               next_event_estimation=False, rr_min_depth=5, max_depth=0, layout=abi.OR3_LAYOUT_REFERENCE,
               seed=0, wave_paths=0, flags=0, tuning=0, callback=None):
        cam = camera.to_c()
        p = self._params(supersamples, min_samples, max_samples, step_samples, next_event_estimation,
                         rr_min_depth, max_depth, layout, seed, wave_paths, flags, tuning)
        if callback is not None:
            def _cb(user, samples, rgb, w, h, minutes):
                img = np.ctypeslib.as_array(rgb, shape=(h, w, 3)).copy()
                callback(samples, img, w, h, minutes)
            cb = abi.FRAME_CB(_cb)
        else:
            cb = abi.FRAME_CB()
        self._check(self.lib.or3_render(self.h, scene, ctypes.byref(cam), ctypes.byref(p), cb, None))
        return self.stats()

    def stop(self):
        self._check(self.lib.or3_stop(self.h))

    def reset_stop(self):
        self._check(self.lib.or3_reset_stop(self.h))

    def stats(self):
        s = abi.RenderStatsC()
        self._check(self.lib.or3_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in abi.RenderStatsC._fields_}

    def frame(self, width, height, layout=abi.OR3_LAYOUT_REFERENCE, out=None):
        """The last frame (2W x H x 3 doubles in the reference layout).  out: a
        C-contiguous float64 array of that shape to fill instead of a new one
        (repeated reads then skip the page faults of a fresh buffer)."""
        w = width * (2 if layout == abi.OR3_LAYOUT_REFERENCE else 1)
        if out is None:
            out = np.zeros((height, w, 3), np.float64)
        elif out.shape != (height, w, 3) or out.dtype != np.float64 or not out.flags.c_contiguous:
            raise ValueError("out must be a C-contiguous float64 array of shape %s" % ((height, w, 3),))
        s = ctypes.c_int32()
        self._check(self.lib.or3_get_frame(self.h, out.ctypes.data_as(abi.f64p), out.size, ctypes.byref(s)))
        return out, s.value

    # ---- image output / input on the device
    def encode_rgb8(self, rgb, gamma=True):
        c = np.ascontiguousarray(rgb, np.float64).reshape(-1, 3)
        out = np.zeros((c.shape[0], 3), np.uint8)
        self._check(self.lib.or3_encode_rgb8(self.h, c.ctypes.data_as(abi.f64p), c.shape[0], 1 if gamma else 0,
                                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return out

    def encode_rgbe(self, rgb):
        c = np.ascontiguousarray(rgb, np.float64).reshape(-1, 3)
        out = np.zeros((c.shape[0], 4), np.uint8)
        self._check(self.lib.or3_encode_rgbe(self.h, c.ctypes.data_as(abi.f64p), c.shape[0],
                                             out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return out

    def decode_rgbe(self, rgbe):
        b = np.ascontiguousarray(rgbe, np.uint8).reshape(-1, 4)
        out = np.zeros((b.shape[0], 3), np.float32)
        self._check(self.lib.or3_decode_rgbe(self.h, b.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), b.shape[0],
                                             out.ctypes.data_as(abi.f32p)))
        return out

    def frame_rgb8(self, width, height, layout=abi.OR3_LAYOUT_REFERENCE, gamma=True):
        w = width * (2 if layout == abi.OR3_LAYOUT_REFERENCE else 1)
        out = np.zeros((height, w, 3), np.uint8)
        s = ctypes.c_int32()
        self._check(self.lib.or3_get_frame_rgb8(self.h, 1 if gamma else 0,
                                                out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), out.size,
                                                ctypes.byref(s)))
        return out, s.value

    def frame_rgbe(self, width, height, layout=abi.OR3_LAYOUT_REFERENCE):
        w = width * (2 if layout == abi.OR3_LAYOUT_REFERENCE else 1)
        out = np.zeros((height, w, 4), np.uint8)
        s = ctypes.c_int32()
        self._check(self.lib.or3_get_frame_rgbe(self.h, out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), out.size,
                                                ctypes.byref(s)))
        return out, s.value

    def moments(self, width, height):
        s = np.zeros((height, width, 3), np.float64)
        q = np.zeros_like(s)
        n = ctypes.c_uint64()
        self._check(self.lib.or3_get_moments(self.h, s.ctypes.data_as(abi.f64p), q.ctypes.data_as(abi.f64p),
                                             s.size, ctypes.byref(n)))
        return s, q, n.value

    def path_radiance(self):
        n = ctypes.c_uint64()
        self._check(self.lib.or3_get_path_radiance(self.h, None, 0, ctypes.byref(n)))
        out = np.zeros((n.value, 3), np.float32)
        self._check(self.lib.or3_get_path_radiance(self.h, out.ctypes.data_as(abi.f32p), out.size, ctypes.byref(n)))
        return out

    # ---- batched form
    def _job(self, scene, camera, settings, frame=None):
        j = abi.BatchJobC()
        j.scene = scene
        j.camera = camera.to_c()
        j.params = self._params(**settings)
        if frame is not None:
            j.frame_host = frame.ctypes.data_as(abi.f64p)
            j.frame_capacity = frame.size
        return j

    def render_batch(self, jobs, *, wave_paths=0, graph_bounces=0, blocks_per_sm=0, flags=0, frames=False):
        """jobs: list of (scene, camera, settings dict).  Returns (stats, frames or None)."""
        n = len(jobs)
        arr = (abi.BatchJobC * n)()
        outs = []
        for k, (sid, cam, st) in enumerate(jobs):
            fr = None
            if frames:
                w = cam.width * (2 if st.get("layout", abi.OR3_LAYOUT_REFERENCE) == abi.OR3_LAYOUT_REFERENCE else 1)
                fr = np.zeros((cam.height, w, 3), np.float64)
                outs.append(fr)
            arr[k] = self._job(sid, cam, st, fr)
        bp = abi.BatchParamsC(wave_paths, flags, graph_bounces, blocks_per_sm, 0)
        s = abi.RenderStatsC()
        self._check(self.lib.or3_render_batch(self.h, arr, n, ctypes.byref(bp), ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in abi.RenderStatsC._fields_}, (outs if frames else None)

    def batch_moments(self, job, width, height):
        s = np.zeros((height, width, 3), np.float64)
        q = np.zeros_like(s)
        n = ctypes.c_uint64()
        self._check(self.lib.or3_get_batch_moments(self.h, job, s.ctypes.data_as(abi.f64p),
                                                   q.ctypes.data_as(abi.f64p), s.size, ctypes.byref(n)))
        return s, q, n.value

    def autotune_batch(self, jobs, sample_paths=1 << 24):
        n = len(jobs)
        arr = (abi.BatchJobC * n)()
        for k, (sid, cam, st) in enumerate(jobs):
            arr[k] = self._job(sid, cam, st)
        best = abi.BatchParamsC()
        rate = ctypes.c_double()
        self._check(self.lib.or3_autotune_batch(self.h, arr, n, sample_paths, ctypes.byref(best), ctypes.byref(rate)))
        return dict(wave_paths=best.wave_paths, graph_bounces=best.graph_bounces,
                    blocks_per_sm=best.blocks_per_sm), rate.value

    # ---- served form
    def server_start(self, *, wave_paths=0, hbm_budget_bytes=0, max_active_jobs=0, frame_every_samples=0,
                     graph_bounces=0, keep_moments=False, on_frame=None, rgb8=False, one_lane=False):
        """rgb8: frames encoded to 8-bit on the device (or3_server_start8); on_frame then
        receives uint8 images.  one_lane: every wave on one stream."""
        p = abi.ServerParamsC(wave_paths, hbm_budget_bytes, max_active_jobs, frame_every_samples, graph_bounces,
                              (abi.OR3_SERVER_KEEP_MOMENTS if keep_moments else 0) |
                              (abi.OR3_SERVER_ONE_LANE if one_lane else 0))
        if rgb8:
            def _cb8(user, job_id, samples, rgb, w, h, final):
                if on_frame is not None:
                    on_frame(job_id, samples, np.ctypeslib.as_array(rgb, shape=(h, w, 3)).copy(), bool(final))
            self._server_cb = abi.JOB_FRAME8_CB(_cb8)
            self._check(self.lib.or3_server_start8(self.h, ctypes.byref(p), self._server_cb, None))
            return
        if on_frame is not None:
            def _cb(user, job_id, samples, rgb, w, h, final):
                on_frame(job_id, samples, np.ctypeslib.as_array(rgb, shape=(h, w, 3)).copy(), bool(final))
            self._server_cb = abi.JOB_FRAME_CB(_cb)
        else:
            self._server_cb = abi.JOB_FRAME_CB()
        self._check(self.lib.or3_server_start(self.h, ctypes.byref(p), self._server_cb, None))

    def server_submit(self, scene, camera, **settings):
        j = self._job(scene, camera, settings)
        jid = ctypes.c_uint64()
        self._check(self.lib.or3_server_submit(self.h, ctypes.byref(j), ctypes.byref(jid)))
        return jid.value

    def server_poll(self, job_id):
        s = abi.JobStatusC()
        self._check(self.lib.or3_server_poll(self.h, job_id, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in abi.JobStatusC._fields_}

    def server_cancel(self, job_id):
        self._check(self.lib.or3_server_cancel(self.h, job_id))

    def server_drain(self, timeout_s=0.0):
        self._check(self.lib.or3_server_drain(self.h, timeout_s))

    def server_stats(self):
        s = abi.ServerStatsC()
        self._check(self.lib.or3_server_get_stats(self.h, ctypes.byref(s)))
        return {k: getattr(s, k) for k, _ in abi.ServerStatsC._fields_}

    def server_moments(self, job_id, width, height):
        s = np.zeros((height, width, 3), np.float64)
        q = np.zeros_like(s)
        n = ctypes.c_uint64()
        self._check(self.lib.or3_server_get_moments(self.h, job_id, s.ctypes.data_as(abi.f64p),
                                                    q.ctypes.data_as(abi.f64p), s.size, ctypes.byref(n)))
        return s, q, n.value

    def server_stop(self):
        self._check(self.lib.or3_server_stop(self.h))

    # ---- ray queries
    def trace_closest(self, scene, origins, dirs):
        o = np.ascontiguousarray(origins, np.float32)
        d = np.ascontiguousarray(dirs, np.float32)
        n = o.shape[0]
        prim = np.zeros(n, np.int32)
        t = np.zeros(n, np.float32)
        nrm = np.zeros((n, 3), np.float32)
        self._check(self.lib.or3_trace_closest(self.h, scene, n, o.ctypes.data_as(abi.f32p),
                                               d.ctypes.data_as(abi.f32p),
                                               prim.ctypes.data_as(ctypes.POINTER(ctypes.c_int32)),
                                               t.ctypes.data_as(abi.f32p), nrm.ctypes.data_as(abi.f32p)))
        return prim, t, nrm

    def env_sample(self, scene, dirs):
        """IBL::Sample per unit direction (n x 3) -> n x 3 float32."""
        d = np.ascontiguousarray(dirs, np.float32).reshape(-1, 3)
        out = np.zeros((d.shape[0], 3), np.float32)
        self._check(self.lib.or3_env_sample(self.h, scene, d.shape[0], d.ctypes.data_as(abi.f32p),
                                            out.ctypes.data_as(abi.f32p)))
        return out

    def texture_sample(self, scene, texture, uv):
        """Image::GetPixelByUV of a scene texture per (u, v) (n x 2) -> n x 3 float32."""
        u = np.ascontiguousarray(uv, np.float32).reshape(-1, 2)
        out = np.zeros((u.shape[0], 3), np.float32)
        self._check(self.lib.or3_texture_sample(self.h, scene, texture, u.shape[0], u.ctypes.data_as(abi.f32p),
                                                out.ctypes.data_as(abi.f32p)))
        return out

    def trace_occluded(self, scene, origins, dirs, tmax):
        o = np.ascontiguousarray(origins, np.float32)
        d = np.ascontiguousarray(dirs, np.float32)
        tm = np.ascontiguousarray(tmax, np.float32)
        occ = np.zeros(o.shape[0], np.uint8)
        self._check(self.lib.or3_trace_occluded(self.h, scene, o.shape[0], o.ctypes.data_as(abi.f32p),
                                                d.ctypes.data_as(abi.f32p), tm.ctypes.data_as(abi.f32p),
                                                occ.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))))
        return occ.astype(bool)


class ScreenPixels:
    """Result view with the reference ScreenPixels accessors (src/renderer/ScreenPixels.hpp:20-71)."""

    def __init__(self, pixels):
        self._px = pixels

    def GetScreen(self):
        return self._px

    def CalcScreenWidth(self):
        return self._px.shape[1]

    def CalcScreenHeight(self):
        return self._px.shape[0]


class GpuPathTracer:
    """Drop-in for PathTracer(camera, min, max, step, supersamples, callback)."""

    def __init__(self, camera, min_samples, max_samples=None, step=1, supersamples=1, callback=None, device=0,
                 context=None):
        if max_samples is None:  # PathTracer(camera, samples, supersamples) form
            max_samples = min_samples
        self.camera = camera
        self.min_samples, self.max_samples, self.step = min_samples, max_samples, step
        self.supersamples = supersamples
        self.callback = callback
        self.ctx = context or Context(device)
        self._nee = False
        self._threads = 1
        self._current = 0
        self._result = None
        self._lock = threading.Lock()
        self.rr_min_depth = 5   # reference MinDepth (src/renderer/PathTracer.cpp:177)
        self.max_depth = 0      # reference: no hard depth limit
        self.seed = 0
        self._scene_cache = {}

    def EnableNextEventEstimation(self, enable=True):
        self._nee = bool(enable)

    def SetMaxThreadCount(self, count):
        # host threads do not apply to the GPU path; kept for interface parity
        self._threads = 1 if count == 0 else int(count)

    def RenderScene(self, scene_desc):
        key = id(scene_desc)
        if key not in self._scene_cache:
            self._scene_cache[key] = self.ctx.upload(scene_desc)
        sid = self._scene_cache[key]

        def on_frame(samples, img, w, h, minutes):
            with self._lock:
                self._current = samples
                self._result = ScreenPixels(img)
            if self.callback:
                self.callback(samples, img, w, h, minutes)

        self.ctx.render(sid, self.camera, supersamples=self.supersamples, min_samples=self.min_samples,
                        max_samples=self.max_samples, step_samples=self.step,
                        next_event_estimation=self._nee, rr_min_depth=self.rr_min_depth,
                        max_depth=self.max_depth, seed=self.seed, callback=on_frame)

    def GetResult(self):
        with self._lock:
            return self._result

    def GetCurrentSampleCount(self):
        return self._current

    def GetCurrentRenderingInfo(self):
        s = self.ctx.stats()
        return ("(width, height) = (%d, %d)\nsamples / pixel = %dx(%dx%d)\npaths = %d, extension rays = %d\n"
                % (self.camera.width, self.camera.height, s["samples"], self.supersamples, self.supersamples,
                   s["camera_paths"], s["extension_rays"]))

    def StopRendering(self):
        self.ctx.stop()


def read_hdr(data):
    """Radiance .hdr file contents (bytes) -> (H, W, 4) uint8 RGBE (or3_read_hdr; host only)."""
    lib = abi.load_library()
    buf = np.frombuffer(bytes(data), np.uint8)
    w, h = ctypes.c_uint32(), ctypes.c_uint32()
    ptr = buf.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8))
    rc = lib.or3_read_hdr(ptr, buf.size, ctypes.byref(w), ctypes.byref(h), None, 0)
    if rc != abi.OR3_OK:
        raise Or3Error(rc, "or3_read_hdr: not a readable Radiance file")
    out = np.zeros((h.value, w.value, 4), np.uint8)
    rc = lib.or3_read_hdr(ptr, buf.size, ctypes.byref(w), ctypes.byref(h),
                          out.ctypes.data_as(ctypes.POINTER(ctypes.c_uint8)), out.size)
    if rc != abi.OR3_OK:
        raise Or3Error(rc, "or3_read_hdr: truncated or malformed pixel data")
    return out


def load_obj(path, flip_v=False, threads=0, position=None, scaling=(1.0, 1.0, 1.0), rotation=(0.0, 0.0, 0.0)):
    """or3_mesh_load_obj (+ or3_mesh_transform when position is given); host only.
    Returns dict: vertices [n,3,3], normals [n,3,3], uvs [n,3,2], material [n],
    materials [(type, colour, ior)], names, textures."""
    lib = abi.load_library()
    mp = ctypes.POINTER(abi.MeshC)()
    rc = lib.or3_mesh_load_obj(str(path).encode(), 1 if flip_v else 0, threads, ctypes.byref(mp))
    if rc != abi.OR3_OK:
        raise Or3Error(rc, "or3_mesh_load_obj(%s) failed" % path)
    try:
        if position is not None:
            d3 = ctypes.c_double * 3
            rc = lib.or3_mesh_transform(mp, d3(*position), d3(*scaling), d3(*rotation))
            if rc != abi.OR3_OK:
                raise Or3Error(rc, "or3_mesh_transform failed")
        m = mp.contents
        n = m.num_triangles
        out = {
            "vertices": np.ctypeslib.as_array(m.vertices, shape=(n, 3, 3)).copy() if n else np.zeros((0, 3, 3)),
            "normals": np.ctypeslib.as_array(m.normals, shape=(n, 3, 3)).copy() if n else np.zeros((0, 3, 3)),
            "uvs": np.ctypeslib.as_array(m.uvs, shape=(n, 3, 2)).copy() if n else np.zeros((0, 3, 2)),
            "material": np.ctypeslib.as_array(m.material, shape=(n,)).copy() if n else np.zeros(0, np.uint32),
            "materials": [(m.materials[i].type, tuple(m.materials[i].color), m.materials[i].ior)
                          for i in range(m.num_materials)],
            "names": [m.material_names[i].decode() for i in range(m.num_materials)],
            "textures": [(m.texture_paths[i].decode() if m.texture_paths[i] else None)
                         for i in range(m.num_materials)],
        }
    finally:
        lib.or3_mesh_free(mp)
    return out


def _scene_file_open(path, threads):
    lib = abi.load_library()
    fp = ctypes.POINTER(abi.SceneFileC)()
    err = ctypes.create_string_buffer(512)
    rc = lib.or3_scene_load_file(str(path).encode(), threads, ctypes.byref(fp), err, len(err))
    if rc != abi.OR3_OK:
        raise Or3Error(rc, "or3_scene_load_file(%s): %s" % (path, err.value.decode(errors="replace")))
    return lib, fp


def scene_from_desc(d):
    """A SceneDesc holding a copy of an or3_scene_desc's arrays (ids kept;
    triangles need their normal, uv and id arrays; textures are not copied)."""
    from .scene import SceneDesc
    sd = SceneDesc()
    for i in range(d.num_materials):
        m = d.materials[i]
        sd.material(m.type, tuple(m.color), tuple(m.emission), m.ior, m.phong_exponent, m.texture)
    sd.layer_material = [d.layer_material[i] for i in range(d.num_layers)]
    sd.layer_rate = [d.layer_rate[i] for i in range(d.num_layers)]
    n = d.num_triangles
    if n:
        arr = np.ctypeslib.as_array
        sd.tris.append((arr(d.tri_vertices, shape=(n, 3, 3)).copy(), arr(d.tri_normals, shape=(n, 3, 3)).copy(),
                        arr(d.tri_uvs, shape=(n, 3, 2)).copy(), arr(d.tri_layers, shape=(n, 2)).copy(),
                        arr(d.tri_ids, shape=(n,)).copy()))
    for i in range(d.num_spheres):
        sd.spheres.append((*(d.spheres[4 * i + k] for k in range(4)), d.sphere_layers[2 * i],
                           d.sphere_layers[2 * i + 1], d.sphere_flags[i] if d.sphere_flags else 0, d.sphere_ids[i]))
    for i in range(d.num_planes):
        sd.planes.append((*(d.planes[4 * i + k] for k in range(4)), d.plane_layers[2 * i],
                          d.plane_layers[2 * i + 1], d.plane_ids[i]))
    sd._next_id = n + d.num_spheres + d.num_planes
    sd.background = tuple(d.background)
    if d.env_rgbe:
        sd.set_env_rgbe(np.ctypeslib.as_array(d.env_rgbe, shape=(d.env_height, d.env_width, 4)).copy())
    elif d.env_rgb:
        sd.set_env(np.ctypeslib.as_array(d.env_rgb, shape=(d.env_height, d.env_width, 3)).copy())
    return sd


def load_scene_file(path, threads=0):
    """The reference's text scene file (SceneFromExternalFile) -> (SceneDesc, info).

    or3_scene_load_file on the host; the arrays are copied into a SceneDesc
    with the file's object ids.  info: space_partitioning, ibl_path, meshes,
    textures (image path per material, or None).
    """
    lib, fp = _scene_file_open(path, threads)
    try:
        f = fp.contents
        d = f.desc
        sd = scene_from_desc(d)
        info = {
            "space_partitioning": f.space_partitioning.decode(),
            "ibl_path": f.ibl_path.decode() if f.ibl_path else None,
            "meshes": f.num_meshes,
            "textures": [(f.texture_paths[i].decode() if f.texture_paths[i] else None)
                         for i in range(d.num_materials)],
        }
    finally:
        lib.or3_scene_file_free(fp)
    return sd, info
