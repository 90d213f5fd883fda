"""Python handle on a native render context (C ABI of include/yapt_gpu.h)."""
import ctypes as C

import numpy as np

from . import _native as N


class Context:
    """Owns one yg_context: device memory, one CUDA stream, the uploaded scene and film."""

    def __init__(self, device=0):
        self.lib = N.load()
        h = C.c_void_p()
        N.check(self.lib.yg_create(N.DATA_DIR.encode(), int(device), C.byref(h)))
        self.h = h
        self.width = self.height = 0

    def close(self):
        if self.h:
            self.lib.yg_destroy(self.h)
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

    # -- scene -------------------------------------------------------------
    def upload_scene(self, scene):
        scene.upload(self.lib, self.h)

    def scene_info(self):
        v = [C.c_uint64() for _ in range(4)]
        N.check(self.lib.yg_scene_info(self.h, *[C.byref(x) for x in v]))
        return dict(triangles=v[0].value, nodes=v[1].value, lights=v[2].value, device_bytes=v[3].value)

    def table(self, name):
        which = N.TABLES[name]
        n = C.c_size_t()
        N.check(self.lib.yg_get_table(self.h, which, None, 0, C.byref(n)))
        dt = np.uint32 if name == "sobol" else np.float32
        out = np.zeros(n.value, dtype=dt)
        if name == "cie":
            out = np.zeros(n.value, dtype=np.float32)
        N.check(self.lib.yg_get_table(self.h, which, out.ctypes.data_as(C.c_void_p), out.size, C.byref(n)))
        return out

    # -- rendering ---------------------------------------------------------
    def film_clear(self, width, height):
        N.check(self.lib.yg_film_clear(self.h, int(width), int(height)))
        self.width, self.height = int(width), int(height)

    @staticmethod
    def params(integrator="nee", width=64, height=64, spp_start=0, spp=1, max_depth=8, regularize_after=8,
               regularize=True, env_scale=0.0, seed=0, flags=0, crop=None, lambda_range=(380.0, 700.0),
               light_paths=0, light_vertices=0):
        p = N.RenderParams()
        p.integrator = N.INTEGRATORS[integrator] if isinstance(integrator, str) else int(integrator)
        p.width, p.height = int(width), int(height)
        p.spp_start, p.spp_count = int(spp_start), int(spp)
        p.max_depth = int(max_depth)
        p.regularize_after_vertices = int(regularize_after)
        p.regularize_enable = 1 if regularize else 0
        p.env_intensity_scale = float(env_scale)
        p.seed = int(seed)
        p.flags = int(flags)
        if crop is not None:
            p.crop_x, p.crop_y, p.crop_w, p.crop_h = [int(v) for v in crop]
        p.lambda_min, p.lambda_max = float(lambda_range[0]), float(lambda_range[1])
        p.bdpt_light_paths = int(light_paths)
        p.bdpt_light_vertices = int(light_vertices)
        return p

    def render(self, params, dump=False):
        """Runs one render request; with dump=True returns the per-sample records
        (spp, crop_h, crop_w, 8): hero lambda, L[4], XYZ."""
        if dump:
            cw = params.crop_w or params.width
            ch = params.crop_h or params.height
            rec = np.zeros((params.spp_count, ch, cw, 8), np.float32)
            N.check(self.lib.yg_render(self.h, C.byref(params), rec.ctypes.data_as(C.c_void_p)))
            return rec
        N.check(self.lib.yg_render(self.h, C.byref(params), None))
        return None

    def synchronize(self):
        N.check(self.lib.yg_synchronize(self.h))

    def film_save(self):
        """The film's state (compensated sums, counts, feature and a-trous accumulators) as bytes."""
        n = C.c_size_t()
        N.check(self.lib.yg_film_state_size(self.h, C.byref(n)))
        buf = (C.c_uint8 * n.value)()
        N.check(self.lib.yg_film_save(self.h, buf, n.value))
        return bytes(buf)

    def film_restore(self, state):
        """Makes a state from film_save this context's film; renders continue its accumulation."""
        buf = (C.c_uint8 * len(state)).from_buffer_copy(state)
        N.check(self.lib.yg_film_restore(self.h, buf, len(state)))
        w, h = np.frombuffer(state[12:20], np.uint32)
        self.width, self.height = int(w), int(h)

    def film(self):
        xyz = np.zeros((self.height, self.width, 3), np.float32)
        cnt = np.zeros((self.height, self.width), np.float32)
        N.check(self.lib.yg_film_read(self.h, xyz.ctypes.data_as(C.POINTER(C.c_float)),
                                      cnt.ctypes.data_as(C.POINTER(C.c_float))))
        return xyz, cnt

    def atrous_denoise(self, params=None):
        """Runs the a-trous denoiser on the film (every film render since film_clear must
        carry YG_FLAG_ATROUS_FEATURES); returns (xyzw (H, W, 4), variance (H, W))."""
        p = params or atrous_params()
        N.check(self.lib.yg_atrous_denoise(self.h, C.byref(p), None, None))
        out = np.zeros((self.height, self.width, 4), np.float32)
        var = np.zeros((self.height, self.width), np.float32)
        N.check(self.lib.yg_atrous_read(self.h, out.ctypes.data_as(C.c_void_p), var.ctypes.data_as(C.c_void_p),
                                        None, None, None, None))
        return out, var

    def tonemap(self, params=None, **kw):
        """The tonemap stage on the film (source 0) or the last a-trous output (source 1):
        returns (RGBA8 (H, W, 4) uint8, the exposure used)."""
        p = params or N.TonemapParams()
        if params is None:
            N.load().yg_tonemap_default_params(C.byref(p))
        for k, v in kw.items():
            if not hasattr(p, k):
                raise ValueError("unknown tonemap parameter %r" % k)
            setattr(p, k, v)
        out = np.zeros((self.height, self.width, 4), np.uint8)
        e = C.c_float()
        N.check(self.lib.yg_tonemap(self.h, C.byref(p), out.ctypes.data_as(C.c_void_p), C.byref(e)))
        return out, e.value

    def atrous_state(self, features=False):
        """The filter's inputs gathered on the device: film sums, odd-sample sums (H, W, 4),
        moment sums (4, H, W, 4) and, after atrous_denoise, the packed features (2, H, W, 4)."""
        H, W = self.height, self.width
        film = np.zeros((H, W, 4), np.float32)
        odd = np.zeros((H, W, 4), np.float32)
        mom = np.zeros((4, H, W, 4), np.float32)
        feat = np.zeros((2, H, W, 4), np.uint32) if features else None
        N.check(self.lib.yg_atrous_read(self.h, None, None, film.ctypes.data_as(C.c_void_p), odd.ctypes.data_as(C.c_void_p),
                                        mom.ctypes.data_as(C.c_void_p),
                                        feat.ctypes.data_as(C.c_void_p) if feat is not None else None))
        return dict(film=film, odd=odd, moments=mom, features=feat)

    def features(self):
        a = np.zeros((self.height, self.width, 3), np.float32)
        n = np.zeros((self.height, self.width, 3), np.float32)
        d = np.zeros((self.height, self.width), np.float32)
        N.check(self.lib.yg_features_read(self.h, a.ctypes.data_as(C.POINTER(C.c_float)),
                                          n.ctypes.data_as(C.POINTER(C.c_float)), d.ctypes.data_as(C.POINTER(C.c_float))))
        return a, n, d

    def relmse(self, reference_xyz, eps=1e-2):
        ref = np.ascontiguousarray(np.asarray(reference_xyz, np.float32))
        out = C.c_double()
        N.check(self.lib.yg_film_relmse(self.h, ref.ctypes.data_as(C.POINTER(C.c_float)), float(eps), C.byref(out)))
        return out.value

    def last_stats(self):
        ms, rays, launches = C.c_float(), C.c_uint64(), C.c_uint32()
        N.check(self.lib.yg_last_render_stats(self.h, C.byref(ms), C.byref(rays), C.byref(launches)))
        return dict(ms=ms.value, rays=rays.value, launches=launches.value)

    def kernel_profile(self):
        """Per-kind device time of the last render made with YG_FLAG_TIME_KERNELS, and (with
        YG_FLAG_COUNT_TRAVERSAL) the traversal work of closest-hit and shadow rays."""
        kp = N.KernelProfile()
        N.check(self.lib.yg_last_kernel_profile(self.h, C.byref(kp)))
        out = {k: {"ms": kp.ms[i], "launches": kp.launches[i]} for i, k in enumerate(N.KERNEL_KINDS)}
        out["connect"] = {"ms": kp.connect_ms, "launches": kp.connect_launches}
        for f in ("closest_rays", "closest_nodes", "closest_triangles", "shadow_rays", "shadow_nodes", "shadow_triangles",
                  "connection_record_bytes"):
            out[f] = getattr(kp, f)
        return out

    def grid_barrier_selftest(self, missing=0, poll_limit=1 << 20):
        """Runs the bounded grid barrier of the persistent serving round once as a cooperative
        kernel whose blocks pass it three times, with `missing` blocks that never arrive.
        Returns (blocks, barriers passed summed over blocks, timed out)."""
        blocks, passes, timed = C.c_uint32(), C.c_uint32(), C.c_uint32()
        N.check(self.lib.yg_grid_barrier_selftest(self.h, int(missing), int(poll_limit), C.byref(blocks),
                                                  C.byref(passes), C.byref(timed)))
        return blocks.value, passes.value, bool(timed.value)

    def traversal_counts(self):
        n, t = C.c_uint64(), C.c_uint64()
        N.check(self.lib.yg_last_traversal_counts(self.h, C.byref(n), C.byref(t)))
        return dict(nodes=n.value, triangles=t.value)


def xyz_to_srgb_linear(xyz):
    """c_srgbXYZToRGB (colorSpaces.hlsl:18-23)."""
    M = np.array([[3.2406, -1.5372, -0.4986], [-0.9689, 1.8758, 0.0415], [0.0557, -0.2040, 1.0570]], np.float32)
    return xyz @ M.T


class Server:
    """The serving loop (yg_server_*): requests on resident scenes, continuous batching.

    contexts: Context objects with scenes built (they stay resident; do not render on them
    directly while the server lives). Options as yg_server_options."""

    def __init__(self, contexts, memory_budget_bytes=0, max_active=0, wave_capacity=0, round_samples=0, max_depth=0,
                 lambda_range=(380.0, 700.0), use_graphs=True, persistent=False, barrier_polls=0):
        self.lib = N.load()
        self.contexts = list(contexts)
        arr = (C.c_void_p * len(self.contexts))(*[c.h.value for c in self.contexts])
        o = N.ServerOptions()
        o.memory_budget_bytes = int(memory_budget_bytes)
        o.max_active = int(max_active)
        o.wave_capacity = int(wave_capacity)
        o.round_samples = int(round_samples)
        o.max_depth = int(max_depth)
        o.lambda_min, o.lambda_max = float(lambda_range[0]), float(lambda_range[1])
        o.use_graphs = 1 if use_graphs else 0
        o.persistent = 1 if persistent else 0
        o.barrier_polls = int(barrier_polls)
        h = C.c_void_p()
        N.check(self.lib.yg_server_create(arr, len(self.contexts), C.byref(o), C.byref(h)))
        self.h = h
        self.sizes = {}

    def close(self):
        if getattr(self, "h", None):
            self.lib.yg_server_destroy(self.h)
            self.h = None

    def __enter__(self):
        return self

    def __exit__(self, *a):
        self.close()

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    def submit(self, scene, params):
        """Queues a request (params from Context.params); returns its id."""
        q = N.Request()
        q.scene = int(scene)
        q.params = params
        rid = C.c_uint64()
        N.check(self.lib.yg_server_submit(self.h, C.byref(q), C.byref(rid)))
        self.sizes[rid.value] = (params.width, params.height)
        return rid.value

    @staticmethod
    def _info(i):
        return dict(state=N.REQ_STATES[i.state], error=i.error, t_submit=i.t_submit, t_admit=i.t_admit, t_done=i.t_done,
                    footprint_bytes=i.footprint_bytes, samples=i.samples)

    def wait(self, rid, timeout=-1.0):
        """Blocks until the request finishes (or timeout seconds); returns its info dict."""
        i = N.RequestInfo()
        rc = self.lib.yg_server_wait(self.h, int(rid), float(timeout), C.byref(i))
        if rc == -4:
            return self._info(i)
        N.check(rc)
        return self._info(i)

    def info(self, rid):
        i = N.RequestInfo()
        N.check(self.lib.yg_server_info(self.h, int(rid), C.byref(i)))
        return self._info(i)

    def result(self, rid):
        w, h = self.sizes[rid]
        xyz = np.zeros((h, w, 3), np.float32)
        cnt = np.zeros((h, w), np.float32)
        N.check(self.lib.yg_server_result(self.h, int(rid), xyz.ctypes.data_as(C.POINTER(C.c_float)),
                                          cnt.ctypes.data_as(C.POINTER(C.c_float))))
        return xyz, cnt

    def cancel(self, rid):
        N.check(self.lib.yg_server_cancel(self.h, int(rid)))

    def release(self, rid):
        N.check(self.lib.yg_server_release(self.h, int(rid)))
        self.sizes.pop(rid, None)

    def stats(self):
        s = N.ServerStats()
        N.check(self.lib.yg_server_stats_get(self.h, C.byref(s)))
        return {k: getattr(s, k) for k, _ in N.ServerStats._fields_}


def plan_round(items, budget_bytes, bytes_in_use=0, max_active=64, wave_capacity=1 << 21, round_samples=1 << 19):
    """One admission + planning decision of the serving loop on host data (yg_server_plan).
    items: dicts with pixels, planes_left, admitted, footprint_bytes, integrator, rounds_waited.
    Returns (admit flags, planes per item, planned samples)."""
    lib = N.load()
    n = len(items)
    arr = (N.SchedItem * max(n, 1))()
    for i, it in enumerate(items):
        arr[i].pixels = int(it["pixels"])
        arr[i].planes_left = int(it["planes_left"])
        arr[i].admitted = 1 if it.get("admitted") else 0
        arr[i].footprint_bytes = int(it.get("footprint_bytes", 0))
        arr[i].integrator = int(N.INTEGRATORS[it["integrator"]] if isinstance(it.get("integrator", 1), str)
                                else it.get("integrator", 1))
        arr[i].rounds_waited = int(it.get("rounds_waited", 0))
    adm = (C.c_uint32 * max(n, 1))()
    pl = (C.c_uint32 * max(n, 1))()
    total = lib.yg_server_plan(arr, n, int(budget_bytes), int(bytes_in_use), int(max_active), int(wave_capacity),
                               int(round_samples), adm, pl)
    if total < 0:
        raise N.YaptError(lib.yg_last_error().decode())
    return [int(adm[i]) for i in range(n)], [int(pl[i]) for i in range(n)], int(total)


def atrous_params(**kw):
    """yg_atrous_params with the reference's defaults, overridden by keyword."""
    p = N.AtrousParams()
    N.load().yg_atrous_default_params(C.byref(p))
    for k, v in kw.items():
        if not hasattr(p, k):
            raise ValueError("unknown a-trous parameter %r" % k)
        setattr(p, k, v)
    return p


def atrous_run(film_sum, odd_sum, moments, camera, params=None):
    """The a-trous filter on host arrays through the C ABI (yg_atrous_run): film_sum, odd_sum
    (H, W, 4) and moments (4, H, W, 4) float32 -> (xyzw, variance, features)."""
    h, w = film_sum.shape[:2]
    f = [np.ascontiguousarray(a, np.float32) for a in (film_sum, odd_sum, moments)]
    out = np.zeros((h, w, 4), np.float32)
    var = np.zeros((h, w), np.float32)
    feat = np.zeros((2, h, w, 4), np.uint32)
    p = params or atrous_params()
    N.check(N.load().yg_atrous_run(w, h, *[a.ctypes.data_as(C.c_void_p) for a in f], C.byref(camera), C.byref(p),
                                   out.ctypes.data_as(C.c_void_p), var.ctypes.data_as(C.c_void_p),
                                   feat.ctypes.data_as(C.c_void_p)))
    return out, var, feat
