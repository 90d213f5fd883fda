"""Learned denoiser: a 4-level U-Net (32/64/128/256 channels, 3x3 convolutions, ReLU) whose
every operator is one of this library's CUDA kernels (yg_nn_* in include/yapt_gpu.h): BF16
tensor-core convolutions with FP32 accumulation for the forward and backward passes, average
pooling, nearest upsampling, the 1x1 RGB head with its relMSE loss, and Adam. PyTorch only
allocates the device buffers and provides the stream.

Input (10 channels, padded to 16): log1p of the linear sRGB radiance of a few-spp render,
albedo, normal, depth. Output: linear sRGB radiance, expm1(input log radiance + the network's
log-space correction), so a clean input passes through. Loss: relMSE, mean (y - t)^2 / (t^2 + eps).

There is no learned denoiser in the reference (its denoiser is the a-trous filter of
postprocess/denoise.comp); this module is the learned part of the serving configuration.
"""
import ctypes as C

import numpy as np

from . import _native as N

# (name, cin, cout, input buffer, output buffer); the buffers are described in UNet._buffers
LAYERS = [
    ("e0a", 16, 32), ("e0b", 32, 32),
    ("e1a", 32, 64), ("e1b", 64, 64),
    ("e2a", 64, 128), ("e2b", 128, 128),
    ("ba", 128, 256), ("bb", 256, 256),
    ("d2a", 384, 128), ("d2b", 128, 128),
    ("d1a", 192, 64), ("d1b", 64, 64),
    ("d0a", 96, 32), ("d0b", 32, 32),
]
HEAD = 3 * 32 + 3
EPS = 0.01  # relMSE epsilon (the film relMSE uses 1e-2 as well)


def _torch():
    import torch
    return torch


def view(t, stride, offset, channels):
    """NHWC view of a device tensor: channel `offset` .. offset + channels of `stride`."""
    return N.NNTensor(t.data_ptr(), stride, offset, channels, 0)


def _check(rc, what):
    if rc != 0:
        raise N.YaptError("%s failed (%d)" % (what, rc))


def parameter_layout():
    """Offsets (in FP32 elements) of every weight and bias in the flat parameter vector, each
    start aligned to 16 elements so that BF16 copies stay 16-byte aligned."""
    lay, o = {}, 0
    for name, cin, cout in LAYERS:
        n = cout * 9 * cin
        lay[name] = (o, n, o + n, cout)  # weight start, weight count, bias start, bias count
        o += n + cout
        o = (o + 15) // 16 * 16
    lay["head"] = (o, 96, o + 96, 3)
    o += HEAD
    o = (o + 15) // 16 * 16
    return lay, o


def init_parameters(seed=0):
    """He-normal weights (fan-in of the 3x3 window), zero biases; head: small normal."""
    lay, n = parameter_layout()
    rng = np.random.Generator(np.random.PCG64(seed))
    p = np.zeros(n, np.float32)
    for name, cin, cout in LAYERS:
        w0, nw, _, _ = lay[name]
        std = np.sqrt(2.0 / (9 * cin))
        if name == "e0a":
            std = np.sqrt(2.0 / (9 * 10))  # 10 of its 16 input channels carry data
        p[w0:w0 + nw] = rng.normal(0.0, std, nw).astype(np.float32)
    h0 = lay["head"][0]
    p[h0:h0 + 96] = rng.normal(0.0, 0.05, 96).astype(np.float32)
    return p


class UNet:
    """U-Net on the device. params: flat FP32 vector (init_parameters layout)."""

    def __init__(self, params=None, device=0, seed=0):
        torch = _torch()
        self.torch = torch
        self.dev = torch.device("cuda", device)
        self.lib = N.load()
        self.lay, self.n = parameter_layout()
        p = init_parameters(seed) if params is None else np.asarray(params, np.float32)
        assert p.size == self.n
        self.p = torch.from_numpy(p.copy()).to(self.dev)
        self.g = torch.zeros_like(self.p)
        self.m = torch.zeros_like(self.p)
        self.v = torch.zeros_like(self.p)
        self.pb = torch.zeros(self.n, dtype=torch.bfloat16, device=self.dev)
        self.wt = torch.zeros(self.n, dtype=torch.bfloat16, device=self.dev)  # flipped weights, same offsets
        self.step_count = 0
        self._sync_bf16()
        self.bufs = {}

    # -- parameters ---------------------------------------------------------
    def stream(self):
        return C.c_void_p(self.torch.cuda.current_stream(self.dev).cuda_stream)

    def _sync_bf16(self):
        self.pb.copy_(self.p.to(self.torch.bfloat16))
        self._flip_all()

    def _flip_all(self):
        for name, cin, cout in LAYERS:
            w0, nw, _, _ = self.lay[name]
            _check(self.lib.yg_nn_flip_weights(C.c_void_p(self.pb.data_ptr() + 2 * w0), cout, cin,
                                               C.c_void_p(self.wt.data_ptr() + 2 * w0), self.stream()), "flip")

    def parameters(self):
        return self.p.detach().cpu().numpy()

    # -- training checkpoints -------------------------------------------------
    def save_checkpoint(self, path):
        """Writes the FP32 weights, both Adam moments and the step count (an .npz file): a run
        restored from it continues with the same updates as the run that wrote it."""
        self.torch.cuda.synchronize(self.dev)
        np.savez(path, params=self.p.cpu().numpy(), adam_m=self.m.cpu().numpy(), adam_v=self.v.cpu().numpy(),
                 step=np.int64(self.step_count), layout=np.int64(self.n))

    @classmethod
    def load_checkpoint(cls, path, device=0):
        z = np.load(path)
        if int(z["layout"]) != parameter_layout()[1]:
            raise ValueError("checkpoint %s: parameter layout of another network" % path)
        net = cls(params=z["params"], device=device)
        net.m.copy_(net.torch.from_numpy(z["adam_m"]).to(net.dev))
        net.v.copy_(net.torch.from_numpy(z["adam_v"]).to(net.dev))
        net.step_count = int(z["step"])
        return net

    # -- buffers ------------------------------------------------------------
    def _buffers(self, n, h, w):
        key = (n, h, w)
        if key in self.bufs:
            return self.bufs[key]
        torch = self.torch
        assert h % 8 == 0 and w % 8 == 0, "image sides must be multiples of 8"
        bf = torch.bfloat16

        def t(ch, s):
            return torch.zeros(n * (h // s) * (w // s) * ch, dtype=bf, device=self.dev)

        B = dict(x0=t(16, 1), e0a=t(32, 1), cat0=t(96, 1), p0=t(32, 2), e1a=t(64, 2), cat1=t(192, 2), p1=t(64, 4),
                 e2a=t(128, 4), cat2=t(384, 4), p2=t(128, 8), ba=t(256, 8), bb=t(256, 8), d2a=t(128, 4),
                 d2b=t(128, 4), d1a=t(64, 2), d1b=t(64, 2), d0a=t(32, 1), d0b=t(32, 1))
        for k in list(B):
            B["g_" + k] = torch.zeros_like(B[k])
        B["out"] = torch.zeros(n * h * w * 3, dtype=torch.float32, device=self.dev)
        self.head_blocks = 152
        B["loss_part"] = torch.zeros(self.head_blocks, dtype=torch.float32, device=self.dev)
        B["gw_part"] = torch.zeros(self.head_blocks * HEAD, dtype=torch.float32, device=self.dev)
        ws = max(self.lib.yg_nn_wgrad_workspace(cin, cout, n, h, w) for _, cin, cout in LAYERS)
        B["ws"] = torch.zeros(ws // 4 + 64, dtype=torch.float32, device=self.dev)
        self.bufs[key] = B
        return B

    # -- operators ----------------------------------------------------------
    def _w(self, name, flipped=False):
        w0 = self.lay[name][0]
        base = self.wt if flipped else self.pb
        return C.c_void_p(base.data_ptr() + 2 * w0)

    def _b(self, name):
        return C.cast(C.c_void_p(self.p.data_ptr() + 4 * self.lay[name][2]), C.POINTER(C.c_float))

    def _conv(self, name, x, y, n, h, w, relu=1, mask=None, acc=0, flipped=False, bias=True):
        rc = self.lib.yg_nn_conv3x3(C.byref(x), self._w(name, flipped), self._b(name) if bias else None, C.byref(y),
                                    C.byref(mask) if mask is not None else None, relu, acc, n, h, w, self.stream())
        _check(rc, "conv " + name)

    def forward(self, x_packed, n, h, w):
        """x_packed: BF16 tensor (n*h*w*16) as built by pack_input; returns FP32 (n*h*w*3)."""
        B = self._buffers(n, h, w)
        B["x0"].copy_(x_packed)
        self._forward(B, n, h, w)
        lib = self.lib
        ho = self.lay["head"]
        hw = C.cast(C.c_void_p(self.p.data_ptr() + 4 * ho[0]), C.POINTER(C.c_float))
        hb = C.cast(C.c_void_p(self.p.data_ptr() + 4 * ho[2]), C.POINTER(C.c_float))
        _check(lib.yg_nn_head(C.byref(view(B["d0b"], 32, 0, 32)), C.byref(view(B["x0"], 16, 0, 16)), hw, hb, n * h * w,
                              C.cast(C.c_void_p(B["out"].data_ptr()), C.POINTER(C.c_float)), None, C.c_float(EPS), None,
                              None, None, self.head_blocks, self.stream()), "head")
        return B["out"]

    def _forward(self, B, n, h, w):
        lib = self.lib
        V = view
        self._conv("e0a", V(B["x0"], 16, 0, 16), V(B["e0a"], 32, 0, 32), n, h, w)
        self._conv("e0b", V(B["e0a"], 32, 0, 32), V(B["cat0"], 96, 64, 32), n, h, w)
        _check(lib.yg_nn_avgpool(C.byref(V(B["cat0"], 96, 64, 32)), C.byref(V(B["p0"], 32, 0, 32)), n, h, w,
                                 self.stream()), "pool0")
        h1, w1 = h // 2, w // 2
        self._conv("e1a", V(B["p0"], 32, 0, 32), V(B["e1a"], 64, 0, 64), n, h1, w1)
        self._conv("e1b", V(B["e1a"], 64, 0, 64), V(B["cat1"], 192, 128, 64), n, h1, w1)
        _check(lib.yg_nn_avgpool(C.byref(V(B["cat1"], 192, 128, 64)), C.byref(V(B["p1"], 64, 0, 64)), n, h1, w1,
                                 self.stream()), "pool1")
        h2, w2 = h // 4, w // 4
        self._conv("e2a", V(B["p1"], 64, 0, 64), V(B["e2a"], 128, 0, 128), n, h2, w2)
        self._conv("e2b", V(B["e2a"], 128, 0, 128), V(B["cat2"], 384, 256, 128), n, h2, w2)
        _check(lib.yg_nn_avgpool(C.byref(V(B["cat2"], 384, 256, 128)), C.byref(V(B["p2"], 128, 0, 128)), n, h2, w2,
                                 self.stream()), "pool2")
        h3, w3 = h // 8, w // 8
        self._conv("ba", V(B["p2"], 128, 0, 128), V(B["ba"], 256, 0, 256), n, h3, w3)
        self._conv("bb", V(B["ba"], 256, 0, 256), V(B["bb"], 256, 0, 256), n, h3, w3)
        _check(lib.yg_nn_upsample(C.byref(V(B["bb"], 256, 0, 256)), C.byref(V(B["cat2"], 384, 0, 256)), n, h3, w3,
                                  self.stream()), "up2")
        self._conv("d2a", V(B["cat2"], 384, 0, 384), V(B["d2a"], 128, 0, 128), n, h2, w2)
        self._conv("d2b", V(B["d2a"], 128, 0, 128), V(B["d2b"], 128, 0, 128), n, h2, w2)
        _check(lib.yg_nn_upsample(C.byref(V(B["d2b"], 128, 0, 128)), C.byref(V(B["cat1"], 192, 0, 128)), n, h2, w2,
                                  self.stream()), "up1")
        self._conv("d1a", V(B["cat1"], 192, 0, 192), V(B["d1a"], 64, 0, 64), n, h1, w1)
        self._conv("d1b", V(B["d1a"], 64, 0, 64), V(B["d1b"], 64, 0, 64), n, h1, w1)
        _check(lib.yg_nn_upsample(C.byref(V(B["d1b"], 64, 0, 64)), C.byref(V(B["cat0"], 96, 0, 64)), n, h1, w1,
                                  self.stream()), "up0")
        self._conv("d0a", V(B["cat0"], 96, 0, 96), V(B["d0a"], 32, 0, 32), n, h, w)
        self._conv("d0b", V(B["d0a"], 32, 0, 32), V(B["d0b"], 32, 0, 32), n, h, w)

    def loss_and_gradients(self, x_packed, target, n, h, w):
        """Forward + backward. target: FP32 (n*h*w*3) linear sRGB. Fills self.g; returns the loss."""
        torch = self.torch
        lib = self.lib
        B = self._buffers(n, h, w)
        B["x0"].copy_(x_packed)
        self._forward(B, n, h, w)
        V = view
        st = self.stream()
        ho = self.lay["head"]
        fp = lambda t, off=0: C.cast(C.c_void_p(t.data_ptr() + 4 * off), C.POINTER(C.c_float))  # noqa: E731
        _check(lib.yg_nn_head(C.byref(V(B["d0b"], 32, 0, 32)), C.byref(V(B["x0"], 16, 0, 16)), fp(self.p, ho[0]),
                              fp(self.p, ho[2]), n * h * w, fp(B["out"]),
                              fp(target), C.c_float(EPS), fp(B["loss_part"]), C.byref(V(B["g_d0b"], 32, 0, 32)),
                              fp(B["gw_part"]), self.head_blocks, st), "head")
        _check(lib.yg_nn_sum_rows(fp(B["gw_part"]), self.head_blocks, HEAD, fp(self.g, ho[0]), st), "head grads")
        ws = C.c_void_p(B["ws"].data_ptr())

        def wgrad(name, x, dy, hh, ww):
            w0, _, b0, _ = self.lay[name]
            _check(lib.yg_nn_conv3x3_wgrad(C.byref(x), C.byref(dy), fp(self.g, w0), fp(self.g, b0), ws, n, hh, ww, st),
                   "wgrad " + name)

        def dgrad(name, dy, dx, hh, ww, mask=None):
            self._conv(name, dy, dx, n, hh, ww, relu=0, mask=mask, flipped=True, bias=False)

        h1, w1, h2, w2, h3, w3 = h // 2, w // 2, h // 4, w // 4, h // 8, w // 8
        # decoder level 0
        wgrad("d0b", V(B["d0a"], 32, 0, 32), V(B["g_d0b"], 32, 0, 32), h, w)
        dgrad("d0b", V(B["g_d0b"], 32, 0, 32), V(B["g_d0a"], 32, 0, 32), h, w, mask=V(B["d0a"], 32, 0, 32))
        wgrad("d0a", V(B["cat0"], 96, 0, 96), V(B["g_d0a"], 32, 0, 32), h, w)
        dgrad("d0a", V(B["g_d0a"], 32, 0, 32), V(B["g_cat0"], 96, 0, 96), h, w)
        _check(lib.yg_nn_upsample_bwd(C.byref(V(B["g_cat0"], 96, 0, 64)), C.byref(V(B["d1b"], 64, 0, 64)),
                                      C.byref(V(B["g_d1b"], 64, 0, 64)), n, h1, w1, st), "up0 bwd")
        # decoder level 1
        wgrad("d1b", V(B["d1a"], 64, 0, 64), V(B["g_d1b"], 64, 0, 64), h1, w1)
        dgrad("d1b", V(B["g_d1b"], 64, 0, 64), V(B["g_d1a"], 64, 0, 64), h1, w1, mask=V(B["d1a"], 64, 0, 64))
        wgrad("d1a", V(B["cat1"], 192, 0, 192), V(B["g_d1a"], 64, 0, 64), h1, w1)
        dgrad("d1a", V(B["g_d1a"], 64, 0, 64), V(B["g_cat1"], 192, 0, 192), h1, w1)
        _check(lib.yg_nn_upsample_bwd(C.byref(V(B["g_cat1"], 192, 0, 128)), C.byref(V(B["d2b"], 128, 0, 128)),
                                      C.byref(V(B["g_d2b"], 128, 0, 128)), n, h2, w2, st), "up1 bwd")
        # decoder level 2
        wgrad("d2b", V(B["d2a"], 128, 0, 128), V(B["g_d2b"], 128, 0, 128), h2, w2)
        dgrad("d2b", V(B["g_d2b"], 128, 0, 128), V(B["g_d2a"], 128, 0, 128), h2, w2, mask=V(B["d2a"], 128, 0, 128))
        wgrad("d2a", V(B["cat2"], 384, 0, 384), V(B["g_d2a"], 128, 0, 128), h2, w2)
        dgrad("d2a", V(B["g_d2a"], 128, 0, 128), V(B["g_cat2"], 384, 0, 384), h2, w2)
        _check(lib.yg_nn_upsample_bwd(C.byref(V(B["g_cat2"], 384, 0, 256)), C.byref(V(B["bb"], 256, 0, 256)),
                                      C.byref(V(B["g_bb"], 256, 0, 256)), n, h3, w3, st), "up2 bwd")
        # bottleneck
        wgrad("bb", V(B["ba"], 256, 0, 256), V(B["g_bb"], 256, 0, 256), h3, w3)
        dgrad("bb", V(B["g_bb"], 256, 0, 256), V(B["g_ba"], 256, 0, 256), h3, w3, mask=V(B["ba"], 256, 0, 256))
        wgrad("ba", V(B["p2"], 128, 0, 128), V(B["g_ba"], 256, 0, 256), h3, w3)
        dgrad("ba", V(B["g_ba"], 256, 0, 256), V(B["g_p2"], 128, 0, 128), h3, w3)
        # encoder level 2
        _check(lib.yg_nn_avgpool_bwd(C.byref(V(B["g_p2"], 128, 0, 128)), C.byref(V(B["g_cat2"], 384, 256, 128)),
                                     C.byref(V(B["cat2"], 384, 256, 128)), C.byref(V(B["g_cat2"], 384, 256, 128)), n, h2,
                                     w2, st), "pool2 bwd")
        wgrad("e2b", V(B["e2a"], 128, 0, 128), V(B["g_cat2"], 384, 256, 128), h2, w2)
        dgrad("e2b", V(B["g_cat2"], 384, 256, 128), V(B["g_e2a"], 128, 0, 128), h2, w2, mask=V(B["e2a"], 128, 0, 128))
        wgrad("e2a", V(B["p1"], 64, 0, 64), V(B["g_e2a"], 128, 0, 128), h2, w2)
        dgrad("e2a", V(B["g_e2a"], 128, 0, 128), V(B["g_p1"], 64, 0, 64), h2, w2)
        # encoder level 1
        _check(lib.yg_nn_avgpool_bwd(C.byref(V(B["g_p1"], 64, 0, 64)), C.byref(V(B["g_cat1"], 192, 128, 64)),
                                     C.byref(V(B["cat1"], 192, 128, 64)), C.byref(V(B["g_cat1"], 192, 128, 64)), n, h1, w1,
                                     st), "pool1 bwd")
        wgrad("e1b", V(B["e1a"], 64, 0, 64), V(B["g_cat1"], 192, 128, 64), h1, w1)
        dgrad("e1b", V(B["g_cat1"], 192, 128, 64), V(B["g_e1a"], 64, 0, 64), h1, w1, mask=V(B["e1a"], 64, 0, 64))
        wgrad("e1a", V(B["p0"], 32, 0, 32), V(B["g_e1a"], 64, 0, 64), h1, w1)
        dgrad("e1a", V(B["g_e1a"], 64, 0, 64), V(B["g_p0"], 32, 0, 32), h1, w1)
        # encoder level 0
        _check(lib.yg_nn_avgpool_bwd(C.byref(V(B["g_p0"], 32, 0, 32)), C.byref(V(B["g_cat0"], 96, 64, 32)),
                                     C.byref(V(B["cat0"], 96, 64, 32)), C.byref(V(B["g_cat0"], 96, 64, 32)), n, h, w, st),
               "pool0 bwd")
        wgrad("e0b", V(B["e0a"], 32, 0, 32), V(B["g_cat0"], 96, 64, 32), h, w)
        dgrad("e0b", V(B["g_cat0"], 96, 64, 32), V(B["g_e0a"], 32, 0, 32), h, w, mask=V(B["e0a"], 32, 0, 32))
        wgrad("e0a", V(B["x0"], 16, 0, 16), V(B["g_e0a"], 32, 0, 32), h, w)
        loss = B["loss_part"].sum().item() / (n * h * w * 3)
        return loss

    def adam_step(self, lr=1e-3, beta1=0.9, beta2=0.999, eps=1e-8):
        self.step_count += 1
        fp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_float))  # noqa: E731
        _check(self.lib.yg_nn_adam(fp(self.p), fp(self.g), fp(self.m), fp(self.v), C.c_void_p(self.pb.data_ptr()), self.n,
                                   C.c_float(lr), C.c_float(beta1), C.c_float(beta2), C.c_float(eps), self.step_count,
                                   self.stream()), "adam")
        self._flip_all()


def pack_input(lib, xyz, albedo, normal, depth, depth_scale, out, stream):
    """Device arrays (FP32, contiguous) -> 16-channel BF16 network input in `out`."""
    fp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_float))  # noqa: E731
    n = depth.numel()
    _check(lib.yg_nn_pack_input(fp(xyz), fp(albedo), fp(normal), fp(depth), C.c_float(depth_scale), n,
                                C.byref(view(out, 16, 0, 16)), stream), "pack")


# ---------------------------------------------------------------------- data and training
SRGB_FROM_XYZ = np.array([[3.2406, -1.5372, -0.4986], [-0.9689, 1.8758, 0.0415], [0.0557, -0.2040, 1.0570]], np.float32)


def render_features(ctx, width, height, spp, spp_start=0, integrator="nee", max_depth=8, lambda_range=(380, 780)):
    """Film mean XYZ and first-hit features of a render on a Context (scene uploaded)."""
    ctx.film_clear(width, height)
    p = ctx.params(integrator, width, height, spp_start=spp_start, spp=spp, max_depth=max_depth, lambda_range=lambda_range,
                   flags=N.YG_FLAG_FEATURES)
    ctx.render(p)
    xyz, _ = ctx.film()
    alb, nrm, dep = ctx.features()
    return xyz, alb, nrm, dep


def render_reference(ctx, width, height, spp, spp_start, integrator="nee", max_depth=8, lambda_range=(380, 780)):
    """Linear sRGB mean of spp samples (sample indices from spp_start)."""
    ctx.film_clear(width, height)
    ctx.render(ctx.params(integrator, width, height, spp_start=spp_start, spp=spp, max_depth=max_depth,
                          lambda_range=lambda_range))
    xyz, _ = ctx.film()
    return xyz @ SRGB_FROM_XYZ.T


def to_device_input(net, xyz, alb, nrm, dep, depth_scale):
    """Host film + features -> packed BF16 input on the device (h*w*16)."""
    torch = net.torch
    h, w = dep.shape
    t = lambda a: torch.from_numpy(np.ascontiguousarray(a, np.float32).reshape(-1)).to(net.dev)  # noqa: E731
    out = torch.zeros(h * w * 16, dtype=torch.bfloat16, device=net.dev)
    pack_input(net.lib, t(xyz), t(alb), t(nrm), t(dep), depth_scale, out, net.stream())
    return out


def relmse(y, ref, eps=EPS):
    y = np.asarray(y, np.float64)
    r = np.asarray(ref, np.float64)
    return float(np.mean((y - r) ** 2 / (r * r + eps)))


def train(net, images, steps, batch=8, crop=128, lr=1e-3, seed=0, log_every=0, lr_final=None):
    """images: list of (packed input (h*w*16 BF16 device tensor), target (h*w*3 FP32 device tensor), h, w).
    Random crops (with flips) per step; Adam on the relMSE loss, the learning rate decaying from lr
    to lr_final on a cosine when lr_final is given. Returns the loss history."""
    torch = net.torch
    rng = np.random.Generator(np.random.PCG64(seed))
    xb = torch.zeros(batch * crop * crop * 16, dtype=torch.bfloat16, device=net.dev)
    tb = torch.zeros(batch * crop * crop * 3, dtype=torch.float32, device=net.dev)
    xv = xb.view(batch, crop, crop, 16)
    tv = tb.view(batch, crop, crop, 3)
    hist = []
    for s in range(steps):
        for b in range(batch):
            x, t, h, w = images[int(rng.integers(len(images)))]
            y0 = int(rng.integers(h - crop + 1))
            x0 = int(rng.integers(w - crop + 1))
            xs = x.view(h, w, 16)[y0:y0 + crop, x0:x0 + crop]
            ts = t.view(h, w, 3)[y0:y0 + crop, x0:x0 + crop]
            if rng.integers(2):
                xs, ts = xs.flip(1), ts.flip(1)
            xv[b].copy_(xs)
            tv[b].copy_(ts)
        loss = net.loss_and_gradients(xb, tb, batch, crop, crop)
        step_lr = lr if lr_final is None else lr_final + 0.5 * (lr - lr_final) * (1.0 + np.cos(np.pi * s / max(1, steps)))
        net.adam_step(step_lr)
        hist.append(loss)
        if log_every and s % log_every == 0:
            print("step %d loss %.5f" % (s, loss), flush=True)
    return hist


class DenoisePipeline:
    """The denoised render on the device: half render A, then B into the same film (so the
    film holds the full mean), the network on A and on the full input, the per-tile error
    estimate ((D(A) - D(full))^2 relative, equal to (D(A) - D(B))^2 / 4 for a linear
    denoiser), and plain accumulation of the worst tiles until the estimated image error fits
    the budget. Film means, features and the packed input never leave the device; only the
    per-tile error estimates (one float a tile) come back to choose the tiles."""

    def __init__(self, net, ctx, height, width, tile=64, depth_scale=4.0):
        torch = net.torch
        self.net, self.ctx, self.h, self.w, self.tile, self.depth_scale = net, ctx, height, width, tile, depth_scale
        n = height * width
        f32 = dict(dtype=torch.float32, device=net.dev)
        self.xyz, self.alb, self.nrm = (torch.zeros(n * 3, **f32) for _ in range(3))
        self.dep = torch.zeros(n, **f32)
        self.packed = torch.zeros(n * 16, dtype=torch.bfloat16, device=net.dev)
        self.den_a = torch.zeros(n * 3, **f32)
        self.tiles = ((height + tile - 1) // tile) * ((width + tile - 1) // tile)
        self.tile_err = torch.zeros(self.tiles, **f32)
        self.tile_flags = torch.zeros(self.tiles, dtype=torch.int32, device=net.dev)

    def _ptr(self, t):
        return C.c_void_p(t.data_ptr())

    def _resolve_and_pack(self):
        lib = self.net.lib
        N.check(lib.yg_film_resolve_device(self.ctx.h, self._ptr(self.xyz), self._ptr(self.alb), self._ptr(self.nrm),
                                           self._ptr(self.dep)))
        fp = lambda t: C.cast(self._ptr(t), C.POINTER(C.c_float))  # noqa: E731
        _check(lib.yg_nn_pack_input(fp(self.xyz), fp(self.alb), fp(self.nrm), fp(self.dep), C.c_float(self.depth_scale),
                                    self.h * self.w, C.byref(view(self.packed, 16, 0, 16)), self.net.stream()), "pack")

    def fallback_tiles(self, target, budget):
        """Tiles to replace by plain accumulation. 4 x tile error estimates the variance part of
        a tile's relMSE; a replaced tile is counted at the target (plain accumulation is run at
        the sample count that reaches it). The worst tiles are replaced until the estimated
        image relMSE is within budget x target; a tile that is not worse than the target is never
        replaced."""
        err = 4.0 * self.tile_err.cpu().numpy().astype(np.float64)
        tx = (self.w + self.tile - 1) // self.tile
        ty = (self.h + self.tile - 1) // self.tile
        npx = np.array([min(self.tile, self.h - (t // tx) * self.tile) * min(self.tile, self.w - (t % tx) * self.tile)
                        for t in range(tx * ty)], np.float64)
        total = float(npx.sum())
        cur = float((err * npx).sum() / total)
        flags = np.zeros(len(err), np.int32)
        for t in np.argsort(-err * npx):
            if cur <= budget * target or err[t] <= target:
                break
            flags[t] = 1
            cur += (target - err[t]) * npx[t] / total
        return flags

    def run(self, spp, spp_plain, target, integrator="uni", max_depth=8, lambda_range=(380, 780), fallback_start=1 << 16,
            budget=0.5):
        """Returns (linear sRGB image h x w x 3 on the host, fallback tile count)."""
        ctx, net, lib, h, w = self.ctx, self.net, self.net.lib, self.h, self.w
        half = max(1, spp // 2)
        kw = dict(max_depth=max_depth, lambda_range=lambda_range, flags=N.YG_FLAG_FEATURES)
        ctx.film_clear(w, h)
        ctx.render(ctx.params(integrator, w, h, spp_start=0, spp=half, **kw))
        self._resolve_and_pack()
        self.den_a.copy_(net.forward(self.packed, 1, h, w))
        net.torch.cuda.current_stream().synchronize()  # the next resolve rewrites the inputs on the context stream
        ctx.render(ctx.params(integrator, w, h, spp_start=half, spp=spp - half, **kw))
        self._resolve_and_pack()
        out = net.forward(self.packed, 1, h, w)
        # threshold / 4: the kernel estimates (a - b)^2 / 4 and here b - a is half of B - A
        _check(lib.yg_nn_tile_error(self._ptr(self.den_a), self._ptr(out), self._ptr(out), h, w, self.tile, C.c_float(EPS),
                                    C.c_float(target / 4.0), self._ptr(self.tile_err), self._ptr(self.tile_flags),
                                    net.stream()), "tile error")
        flags = self.fallback_tiles(target, budget)
        self.tile_flags.copy_(net.torch.from_numpy(flags))
        bad = np.nonzero(flags)[0]
        if len(bad):
            tx = (w + self.tile - 1) // self.tile
            ctx.film_clear(w, h)
            for t in bad:
                y0, x0 = (int(t) // tx) * self.tile, (int(t) % tx) * self.tile
                ctx.render(ctx.params(integrator, w, h, spp_start=fallback_start, spp=spp_plain,
                                      crop=(x0, y0, min(self.tile, w - x0), min(self.tile, h - y0)),
                                      max_depth=max_depth, lambda_range=lambda_range))
            N.check(lib.yg_film_resolve_device(ctx.h, self._ptr(self.xyz), None, None, None))
            _check(lib.yg_nn_tile_fallback(self._ptr(out), self._ptr(self.xyz), self._ptr(self.tile_flags), h, w, self.tile,
                                           net.stream()), "tile fallback")
        return out.view(h, w, 3).cpu().numpy(), int(len(bad))


def denoise_image(net, packed, h, w):
    """Runs the network on a whole image (sides multiples of 8); returns host linear sRGB (h, w, 3)."""
    out = net.forward(packed, 1, h, w)
    return out.view(h, w, 3).cpu().numpy()


def _profile_forward(width, height, reps):
    """U-Net forward passes on a synthetic input (for timing and kernel profiles)."""
    torch = _torch()
    net = UNet(seed=0)
    rng = np.random.Generator(np.random.PCG64(0))
    x = torch.from_numpy(rng.uniform(0, 1, width * height * 16).astype(np.float32)).cuda().to(torch.bfloat16)
    for _ in range(reps):
        net.forward(x, 1, height, width)
    torch.cuda.synchronize()
    e0, e1 = torch.cuda.Event(enable_timing=True), torch.cuda.Event(enable_timing=True)
    e0.record()
    net.forward(x, 1, height, width)
    e1.record()
    torch.cuda.synchronize()
    print("forward %dx%d: %.3f ms" % (width, height, e0.elapsed_time(e1)))


if __name__ == "__main__":
    import argparse
    ap = argparse.ArgumentParser(description="U-Net forward timing on a synthetic input")
    ap.add_argument("--width", type=int, default=1920)
    ap.add_argument("--height", type=int, default=1080)
    ap.add_argument("--reps", type=int, default=3)
    ap.add_argument("--impl", default="tcgen05_tma", choices=["tcgen05", "tcgen05_tma", "mma_sync"])
    a = ap.parse_args()
    impls = {"tcgen05": N.YG_NN_CONV_TCGEN05, "tcgen05_tma": N.YG_NN_CONV_TCGEN05_TMA, "mma_sync": N.YG_NN_CONV_MMA_SYNC}
    N.check(N.load().yg_nn_set_conv_impl(impls[a.impl]))
    _profile_forward(a.width, a.height, a.reps)
