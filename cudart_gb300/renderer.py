"""Host-side mirror of CudaRT's renderer interface over the GB300 C ABI.

`GB300Renderer` follows the reference's abstract `Renderer`
(src/include/renderer.h:78-100): construct it with a scene, width, height
and samples; call `render_one_sample_per_pixel()` once per pass (or
`render(n)`), then `copy_image_bytes()` for the gamma-corrected RGBA8 image
(parallel_renderer.cu:303-310).  `GB300Scene` wraps the scene handle and the
batched closest-hit query.
"""
from __future__ import annotations

import ctypes as C
from typing import Optional

import numpy as np

from . import _lib
from ._lib import (Camera, Material, RenderOptions, SceneDesc, SceneInfo, TuneParams, TuneResult,
                   View, check, load)
from .scenes import NO_TEXTURE, SceneArrays

NODE_DT = np.dtype([("p", "<f4", 3), ("e", "u1", 3), ("imask", "u1"), ("child_base", "<u4"),
                    ("tri_base", "<u4"), ("meta", "u1", 8), ("qlo", "u1", (3, 8)),
                    ("qhi", "u1", (3, 8))])
TRI_DT = np.dtype([("v1", "<f4", 3), ("face", "<u4"), ("e1", "<f4", 3), ("pad1", "<f4"),
                   ("e2", "<f4", 3), ("pad2", "<f4")])
assert NODE_DT.itemsize == 80 and TRI_DT.itemsize == 48


def _ptr(a: np.ndarray):
    return a.ctypes.data_as(C.c_void_p)


def camera_from_json(spec, width: int, height: int) -> Camera:
    """CameraJsonLoader::getCamera (json_loader.cpp:26-48) for a CameraSpec."""
    cam = Camera()
    f3 = lambda v: np.ascontiguousarray(v, np.float32)
    eye, vd, up = f3(spec.eye), f3(spec.view_dir), f3(spec.up)
    check(load().crt_camera_from_json(spec.fov_deg, spec.focal_length, spec.fstop, _ptr(eye),
                                      _ptr(vd), _ptr(up), width, height, C.byref(cam)))
    return cam


def bvh_build_host(positions: np.ndarray, width: int = 8):
    """Host-only BVH build (4 or 8 children per node): (nodes, triangle
    records, max depth)."""
    pos = np.ascontiguousarray(positions, np.float32).reshape(-1, 9)
    n = len(pos)
    nn, depth = C.c_uint32(0), C.c_uint32(0)
    L = load()
    check(L.crt_bvh_build_host(_ptr(pos), n, width, C.byref(nn), C.byref(depth), None, None))
    nodes = np.zeros(nn.value, NODE_DT)
    tris = np.zeros(n, TRI_DT)
    check(L.crt_bvh_build_host(_ptr(pos), n, width, C.byref(nn), C.byref(depth), _ptr(nodes),
                               _ptr(tris)))
    return nodes, tris, depth.value


NODE_FORMATS = {"q8": _lib.NODES_Q8, "f32": _lib.NODES_F32}


def _rgba8(img: np.ndarray) -> np.ndarray:
    """uint8 [h, w, 3 or 4] image -> flat RGBA8 bytes."""
    img = np.asarray(img, np.uint8)
    if img.shape[2] == 3:
        img = np.concatenate([img, np.full(img.shape[:2] + (1,), 255, np.uint8)], axis=2)
    return np.ascontiguousarray(img[..., :4]).reshape(-1)


def _face_areas(e1: np.ndarray, e2: np.ndarray) -> np.ndarray:
    """|e1 x e2| / 2 per face in float32, each operation rounded like the
    reference's Scene::loadTriangles (length(cross(e1, e2)) / 2)."""
    cx = e1[:, 1] * e2[:, 2] - e1[:, 2] * e2[:, 1]
    cy = e1[:, 2] * e2[:, 0] - e1[:, 0] * e2[:, 2]
    cz = e1[:, 0] * e2[:, 1] - e1[:, 1] * e2[:, 0]
    return np.sqrt(cx * cx + cy * cy + cz * cz) / np.float32(2.0)


def _material_table(materials, kd=None, ka=None):
    """crt_material array; kd / ka ([n, 3]) override the materials' values."""
    mats = (Material * len(materials))()
    for i, m in enumerate(materials):
        mats[i].bsdf = m.bsdf
        mats[i].texture = m.tex if m.tex is not None else NO_TEXTURE
        mats[i].kd[:] = list(map(float, m.kd if kd is None else kd[i]))
        mats[i].ka[:] = list(map(float, m.ka if ka is None else ka[i]))
        mats[i].ks[:] = list(map(float, m.ks))
        mats[i].ns, mats[i].ni, mats[i].diffuse = m.ns, m.ni, m.diffuse
    return mats


class GB300Scene:
    """Scene handle: BVH, triangles, materials, lights and textures on the GPU."""

    def __init__(self, sc, lights: Optional[np.ndarray] = None,
                 node_format: str = "q8", bvh_width: int = 8, reference_layout: bool = False,
                 builder: str = "host"):
        """sc: SceneArrays, or ingest.SceneFiles (a scene read from OBJ/MTL/PNG
        files by the library's loader).

        reference_layout: pass the arrays the way the reference's Scene
        holds them after construction (CRT_SCENE_EDGES | CRT_SCENE_KA_SCALED:
        v1/e1/e2 per face, emission already multiplied by 3 x light area),
        which is what the C++ Renderer shim sends."""
        L = load()
        self.arrays = sc
        self.node_format = node_format
        self.bvh_width = bvh_width
        builder_id = {"host": _lib.BVH_HOST, "gpu": _lib.BVH_GPU}[builder]
        from .ingest import SceneFiles
        if isinstance(sc, SceneFiles):
            # straight from the loader's buffers (face-order emissive lights)
            if reference_layout or lights is not None:
                raise ValueError("a SceneFiles scene takes neither lights nor reference_layout")
            desc = sc.desc()
            desc.node_format, desc.bvh_width, desc.builder = NODE_FORMATS[node_format], bvh_width, builder_id
            h = C.c_void_p()
            check(L.crt_scene_create(C.byref(desc), C.byref(h)))
            self.handle = h
            return
        self._keep = []
        pos = np.ascontiguousarray(sc.positions, np.float32)
        nor = np.ascontiguousarray(sc.normals, np.float32)
        uvs = np.ascontiguousarray(sc.uvs, np.float32)
        mid = np.ascontiguousarray(sc.material_ids, np.uint32)
        flags = 0
        if reference_layout:
            p = pos.reshape(-1, 3, 3)
            e1, e2 = p[:, 1] - p[:, 0], p[:, 2] - p[:, 0]
            pos = np.ascontiguousarray(np.stack([p[:, 0], e1, e2], axis=1))
            area = _face_areas(e1, e2)
            order = lights if lights is not None else sc.light_indices()
            lights_area = np.float32(0)
            for f in order:                          # float32, in pick order
                lights_area = np.float32(lights_area + area[f])
            ka = np.array([m.ka for m in sc.materials], np.float32)
            ka = (ka * np.float32(3.0)) * lights_area
            mats = _material_table(sc.materials, ka=ka)
            flags = _lib.SCENE_EDGES | _lib.SCENE_KA_SCALED
        else:
            mats = _material_table(sc.materials)
        dims = np.asarray([d for img in sc.textures for d in (img.shape[1], img.shape[0])], np.uint32)
        # RGBA8 texels, converted on the device as stbi_loadf converts them
        if len(sc.textures) == 1:
            rgba = _rgba8(sc.textures[0])          # a view: no copy of the caller's (maybe pinned) bytes
        elif sc.textures:
            rgba = np.concatenate([_rgba8(img) for img in sc.textures])
        else:
            rgba = np.zeros(4, np.uint8)
        li = (np.ascontiguousarray(lights, np.uint32) if lights is not None
              else np.zeros(1, np.uint32))
        self._keep += [pos, nor, uvs, mid, mats, dims, rgba, li]
        desc = SceneDesc(sc.n_tris, pos.ctypes.data, nor.ctypes.data, uvs.ctypes.data,
                         mid.ctypes.data, len(sc.materials), C.addressof(mats),
                         len(lights) if lights is not None else 0,
                         li.ctypes.data if lights is not None else None,
                         len(sc.textures), dims.ctypes.data if len(dims) else None,
                         None, NODE_FORMATS[node_format], bvh_width, flags, builder_id,
                         rgba.ctypes.data if sc.textures else None)
        h = C.c_void_p()
        check(L.crt_scene_create(C.byref(desc), C.byref(h)))
        self.handle = h
        self._keep = None

    def __del__(self):
        if getattr(self, "handle", None):
            load().crt_scene_destroy(self.handle)
            self.handle = None

    @property
    def info(self) -> SceneInfo:
        inf = SceneInfo()
        check(load().crt_scene_get_info(self.handle, C.byref(inf)))
        return inf

    def set_materials(self, kd=None, ka=None) -> None:
        """Replace every material's kd and/or ka ([num_materials, 3] arrays;
        None keeps the scene's original values)."""
        mats = _material_table(self.arrays.materials, kd, ka)
        check(load().crt_scene_set_materials(self.handle, mats, len(mats)))

    def set_visit_limit(self, max_visits: int) -> None:
        """Node visits a traversal may make before the watchdog ends it (0 = default)."""
        check(load().crt_scene_set_visit_limit(self.handle, max_visits))

    def clear_errors(self) -> None:
        """Reset the scene's sticky device error word (after CRT_ERR_WATCHDOG)."""
        check(load().crt_scene_clear_errors(self.handle))

    def errors(self, stream: Optional[int] = None) -> int:
        """The scene's sticky device error word (SCENE_ERR_* bits) after the
        work queued on `stream` (default: the default stream)."""
        bits = C.c_uint32(0)
        check(load().crt_scene_errors(self.handle, stream, C.byref(bits)))
        return int(bits.value)

    def set_bvh_width(self, width: int) -> None:
        """Rebuild the BVH with 4 or 8 children per node (same geometry)."""
        check(load().crt_scene_set_bvh_width(self.handle, width))
        self.bvh_width = width

    def export_bvh(self):
        inf = self.info
        nodes = np.zeros(inf.num_nodes, NODE_DT)
        tris = np.zeros(inf.num_triangles, TRI_DT)
        check(load().crt_scene_export_bvh(self.handle, _ptr(nodes), _ptr(tris)))
        return nodes, tris

    def trace_closest(self, rays, stream=None):
        """rays: CUDA float32 tensor [n, 8] -> (face int32, t float32, uv float32 [n,2])."""
        import torch
        rays = rays.contiguous()
        n = rays.shape[0]
        idx = torch.empty(n, dtype=torch.int32, device=rays.device)
        t = torch.empty(n, dtype=torch.float32, device=rays.device)
        uv = torch.empty((n, 2), dtype=torch.float32, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream(rays.device).cuda_stream
        check(load().crt_trace_closest(self.handle, rays.data_ptr(), n, idx.data_ptr(), t.data_ptr(),
                                       uv.data_ptr(), s))
        return idx, t, uv

    def trace_counts(self, rays, stream=None):
        import torch
        rays = rays.contiguous()
        n = rays.shape[0]
        nodes = torch.empty(n, dtype=torch.int32, device=rays.device)
        tris = torch.empty(n, dtype=torch.int32, device=rays.device)
        s = stream if stream is not None else torch.cuda.current_stream(rays.device).cuda_stream
        check(load().crt_trace_counts(self.handle, rays.data_ptr(), n, nodes.data_ptr(),
                                      tris.data_ptr(), s))
        return nodes, tris


def make_options(max_depth: int = 6, seed: int = 1234, mode: str = "megakernel", view_id: int = 0,
                 wave_paths: int = 0, flags: int = 0, wave_sets: int = 0, block_size: int = 0,
                 stack_depth: int = 0, node_format: Optional[str] = None, queue_chunk: int = 0,
                 top_nodes: int = 9, refill_busy: int = 0,
                 options: Optional[RenderOptions] = None) -> RenderOptions:
    """crt_render_options from keywords; `options` (e.g. the autotuner's
    choice) overrides them all."""
    if options is not None:
        return options
    opts = RenderOptions()
    load().crt_render_options_default(C.byref(opts))
    opts.max_depth = max_depth
    opts.seed = seed
    opts.view_id = view_id
    opts.mode = {"megakernel": _lib.MODE_MEGAKERNEL, "wavefront": _lib.MODE_WAVEFRONT}[mode]
    opts.wave_paths = wave_paths
    opts.flags = flags
    opts.wave_sets = wave_sets
    opts.block_size = block_size
    opts.stack_depth = stack_depth
    opts.node_format = -1 if node_format is None else NODE_FORMATS[node_format]
    opts.queue_chunk = queue_chunk
    opts.top_nodes = top_nodes
    opts.refill_busy = refill_busy
    return opts


class GB300Renderer:
    """Drop-in for ParallelRenderer (renderer.h:102-126) over the C ABI."""

    def __init__(self, scene: GB300Scene, width: int, height: int, samples: int,
                 camera: Optional[Camera] = None, max_depth: int = 6, seed: int = 1234,
                 mode: str = "megakernel", view_id: int = 0, wave_paths: int = 0,
                 flags: int = 0, wave_sets: int = 0, block_size: int = 0,
                 stack_depth: int = 0, node_format: Optional[str] = None,
                 queue_chunk: int = 0, top_nodes: int = 9, refill_busy: int = 0,
                 options: Optional[RenderOptions] = None):
        L = load()
        self.scene = scene
        self.width, self.height, self.samples = width, height, samples
        if camera is None:
            camera = camera_from_json(scene.arrays.camera, width, height)
        self.camera = camera
        opts = make_options(max_depth, seed, mode, view_id, wave_paths, flags, wave_sets,
                            block_size, stack_depth, node_format, queue_chunk, top_nodes, refill_busy,
                            options)
        self.options = opts
        h = C.c_void_p()
        check(L.crt_render_create(scene.handle, C.byref(camera), width, height, C.byref(opts),
                                  C.byref(h)))
        self.handle = h

    def __del__(self):
        if getattr(self, "handle", None):
            load().crt_render_destroy(self.handle)
            self.handle = None

    # Renderer interface (renderer.h:83-91)
    def render_one_sample_per_pixel(self) -> None:
        check(load().crt_render_pass(self.handle, 1))

    def render(self, n_spp: Optional[int] = None) -> None:
        check(load().crt_render_pass(self.handle, self.samples if n_spp is None else n_spp))

    def copy_image_bytes(self, out: Optional[np.ndarray] = None) -> np.ndarray:
        """RGBA8 [h, w, 4] (crt_render_resolve); `out` (e.g. pinned) is filled if given."""
        if out is None:
            out = np.zeros((self.height, self.width, 4), np.uint8)
        elif out.shape != (self.height, self.width, 4) or out.dtype != np.uint8 or not out.flags["C_CONTIGUOUS"]:
            raise ValueError("out must be a contiguous uint8 [height, width, 4] array")
        check(load().crt_render_resolve(self.handle, _ptr(out)))
        return out

    def get_width(self) -> int:
        return self.width

    def get_height(self) -> int:
        return self.height

    def get_samples(self) -> int:
        return self.samples

    def get_samples_rendered(self) -> int:
        v = C.c_uint32(0)
        check(load().crt_render_samples_rendered(self.handle, C.byref(v)))
        return v.value

    # extensions
    def accum(self) -> np.ndarray:
        out = np.zeros((self.height * self.width, 3), np.float32)
        check(load().crt_render_accum(self.handle, _ptr(out)))
        return out

    def accum_device_ptr(self) -> int:
        p = C.c_void_p()
        check(load().crt_render_accum_device(self.handle, C.byref(p)))
        return p.value

    def accum_tensor(self):
        """The device accumulator as a torch CUDA tensor [height*width, 4]
        (rgb + unused), without a copy; valid while the handle lives.  Lets
        the ranks of a sample-sharded render sum their accumulators in place
        (cudart_gb300.sharding.reduce_accumulators)."""
        import torch
        ptr = self.accum_device_ptr()
        n = self.height * self.width

        class _View:
            __cuda_array_interface__ = {"shape": (n, 4), "typestr": "<f4", "data": (ptr, False),
                                        "version": 2, "strides": None}
        return torch.as_tensor(_View(), device="cuda")

    def synchronize(self) -> None:
        check(load().crt_render_synchronize(self.handle))

    def reset(self) -> None:
        check(load().crt_render_reset(self.handle))

    def load_accum(self, rgb: np.ndarray, samples: int, first_sample: int = 0) -> None:
        """Resume: install FP32 sums of `samples` samples that started at
        `first_sample` ([h*w, 3]); the next pass continues after them."""
        a = np.ascontiguousarray(rgb, np.float32).reshape(-1, 3)
        check(load().crt_render_load_accum(self.handle, 0, _ptr(a), samples, first_sample))

    def resolve_async(self, pinned_u8) -> None:
        """Queue resolve + copy into a pinned host buffer (torch uint8 tensor
        with pin_memory=True, h*w*4 bytes); valid after synchronize()."""
        check(load().crt_render_resolve_async(self.handle, pinned_u8.data_ptr()))

    def restart(self, first_sample: int) -> None:
        """Empty accumulator; the next pass starts at sample first_sample."""
        check(load().crt_render_restart(self.handle, first_sample))

    def set_camera(self, camera: Camera) -> None:
        check(load().crt_render_set_camera(self.handle, C.byref(camera)))
        self.camera = camera

    def set_stream(self, stream: int) -> None:
        check(load().crt_render_set_stream(self.handle, stream))

    def profile_pass(self, n_spp: int) -> dict:
        """Wavefront pass with per-stage CUDA-event timing and traversal counts."""
        p = _lib.StageProfile()
        check(load().crt_render_profile_pass(self.handle, n_spp, C.byref(p)))
        out = {f"{s}_ms": p.ms[i] for i, s in enumerate(p.STAGES)}
        out.update({f"{s}_launches": p.launches[i] for i, s in enumerate(p.STAGES)})
        for f in ("extension_rays", "extension_nodes", "extension_tris", "shadow_rays",
                  "shadow_nodes", "shadow_tris", "extension_top_nodes", "shadow_top_nodes"):
            out[f] = getattr(p, f)
        for f in ("extend_ms_by_bounce", "extend_rays_by_bounce", "shadow_ms_by_bounce",
                  "shadow_rays_by_bounce"):
            out[f] = list(getattr(p, f))
        return out

    def ray_counts(self):
        e, s = C.c_uint64(0), C.c_uint64(0)
        check(load().crt_render_ray_counts(self.handle, C.byref(e), C.byref(s)))
        return e.value, s.value

    def adjoint(self, spp0: int, n_spp: int, adjoint_ptr: int, grad_kd_ptr: int, grad_ka_ptr: int,
                exact_roulette: bool = False) -> None:
        """Path-replay adjoint over device buffers (see crt_render_adjoint):
        adds d<adjoint, radiance sum of samples [spp0, spp0+n_spp)>/d(kd, ka)
        to the [num_materials][3] float buffers.  Runs on the handle's stream
        (synchronize() before reading the gradients)."""
        flags = _lib.ADJOINT_EXACT_ROULETTE if exact_roulette else 0
        check(load().crt_render_adjoint(self.handle, spp0, n_spp, adjoint_ptr, grad_kd_ptr, grad_ka_ptr,
                                        flags))


class GB300Batch:
    """Many camera views of one scene rendered together (crt_batch_*).
    `views`: scenes.View items (camera spec, width, height, spp); view k uses
    Philox view word view_ids[k] (default k)."""

    def __init__(self, scene: GB300Scene, views, view_ids=None, **kw):
        L = load()
        self.scene = scene
        self.views = list(views)
        n = len(self.views)
        arr = (View * n)()
        for k, v in enumerate(self.views):
            arr[k].camera = camera_from_json(v.camera, v.width, v.height)
            arr[k].width, arr[k].height, arr[k].spp = v.width, v.height, v.spp
            arr[k].view_id = k if view_ids is None else int(view_ids[k])
        self._descs = arr
        self.options = make_options(**kw)
        h = C.c_void_p()
        check(L.crt_batch_create(scene.handle, arr, n, C.byref(self.options), C.byref(h)))
        self.handle = h

    def __del__(self):
        if getattr(self, "handle", None):
            load().crt_render_destroy(self.handle)
            self.handle = None

    def __len__(self):
        return len(self.views)

    def render(self) -> None:
        """Every view's own spp."""
        check(load().crt_batch_render(self.handle))

    def render_pass(self, n_spp: int) -> None:
        check(load().crt_render_pass(self.handle, n_spp))

    def synchronize(self) -> None:
        check(load().crt_render_synchronize(self.handle))

    def view_info(self, k: int):
        d, s, off = View(), C.c_uint32(0), C.c_uint32(0)
        check(load().crt_render_view_info(self.handle, k, C.byref(d), C.byref(s), C.byref(off)))
        return dict(width=d.width, height=d.height, spp=d.spp, view_id=d.view_id,
                    samples_rendered=s.value, pixel_offset=off.value)

    def accum(self, k: int) -> np.ndarray:
        v = self.views[k]
        out = np.zeros((v.height * v.width, 3), np.float32)
        check(load().crt_render_view_accum(self.handle, k, _ptr(out)))
        return out

    def resolve(self, k: int) -> np.ndarray:
        v = self.views[k]
        out = np.zeros((v.height, v.width, 4), np.uint8)
        check(load().crt_render_view_resolve(self.handle, k, _ptr(out)))
        return out

    def set_stream(self, stream: int) -> None:
        check(load().crt_render_set_stream(self.handle, stream))

    def ray_counts(self):
        e, s = C.c_uint64(0), C.c_uint64(0)
        check(load().crt_render_ray_counts(self.handle, C.byref(e), C.byref(s)))
        return e.value, s.value


def autotune(scene: GB300Scene, width: int, height: int, camera: Optional[Camera] = None,
             max_depth: int = 6, seed: int = 1234, trial_spp: int = 8, repeats: int = 3,
             rounds: int = 2, tune_bvh_width: bool = True, start: Optional[RenderOptions] = None):
    """Time short wavefront renders of this workload and return the fastest
    launch options (a TuneResult; pass ``result.options`` to GB300Renderer).
    With ``tune_bvh_width`` the scene's BVH may be rebuilt 4-wide."""
    L = load()
    if camera is None:
        camera = camera_from_json(scene.arrays.camera, width, height)
    if start is None:
        start = RenderOptions()
        L.crt_render_options_default(C.byref(start))
        start.max_depth = max_depth
        start.seed = seed
    p = TuneParams()
    L.crt_tune_params_default(C.byref(p))
    p.trial_spp, p.repeats, p.rounds, p.tune_bvh_width = trial_spp, repeats, rounds, int(tune_bvh_width)
    res = TuneResult()
    check(L.crt_autotune(scene.handle, C.byref(camera), width, height, C.byref(start), C.byref(p),
                         C.byref(res)))
    scene.bvh_width = res.bvh_width
    return res


def options_dict(o: RenderOptions) -> dict:
    return {name: getattr(o, name) for name, _ in o._fields_}


def measure_gather(buf, record_bytes: int, n_threads: int, loads_per_thread: int, l1: bool = False,
                   stream: Optional[int] = None):
    """Queue one gather-ceiling launch (crt_measure_gather) over the CUDA
    tensor `buf`: n_threads threads each fetch loads_per_thread records of
    record_bytes from pseudo-random record indices, through L2 only or
    (l1=True) through L1.  Returns the sink tensor; the bytes fetched are
    n_threads * loads_per_thread * record_bytes.  Time it with events on
    `stream` (default: the current stream)."""
    import torch
    sink = torch.empty(n_threads, dtype=torch.int32, device=buf.device)
    s = stream if stream is not None else torch.cuda.current_stream(buf.device).cuda_stream
    check(load().crt_measure_gather(buf.data_ptr(), buf.numel() * buf.element_size(), record_bytes,
                                    n_threads, loads_per_thread, _lib.GATHER_L1 if l1 else 0,
                                    sink.data_ptr(), s))
    return sink
