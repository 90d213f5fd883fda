"""Denoiser kernels against the CPU oracle (oracle/unet_ref.py, float64 with the same BF16
rounding points), the whole U-Net's loss and gradients against the oracle (gradient check),
and a short training run that must beat the noisy input it starts from.

Tolerances: operator outputs stored in BF16 may differ by one BF16 rounding of an FP32 sum
that was accumulated in another order (relative 2^-7); weight gradients accumulate BF16
products in FP32 (relative 1e-3 of the gradient's norm); network gradients per layer: cosine
similarity >= 0.999 and norms within 2%.
"""
import numpy as np
import pytest

pytestmark = pytest.mark.gpu


@pytest.fixture(scope="module")
def torch_cuda(built):
    torch = pytest.importorskip("torch")
    return torch


def dev_bf16(torch, a):
    return torch.from_numpy(np.ascontiguousarray(a, np.float32)).to("cuda").to(torch.bfloat16)


def host(t):
    return t.float().cpu().numpy()


def stream(torch):
    import ctypes as C
    return C.c_void_p(torch.cuda.current_stream().cuda_stream)


IMPLS = {"mma_sync": 0, "tcgen05": 1, "tcgen05_tma": 2}


@pytest.fixture(params=list(IMPLS))
def conv_impl(request, torch_cuda):
    """Runs a test with each tensor-core path of yg_nn_conv3x3, then restores the default."""
    from yapt_gb300 import _native as N
    lib = N.load()
    assert lib.yg_nn_set_conv_impl(IMPLS[request.param]) == 0
    yield request.param
    torch_cuda.cuda.synchronize()
    import ctypes as C
    t = C.c_uint32()
    assert lib.yg_nn_tc_timeouts(C.byref(t)) == 0 and t.value == 0, "tcgen05 waits ran out"
    assert lib.yg_nn_set_conv_impl(0) == 0


@pytest.mark.parametrize("cin,cout,off", [(16, 32, 0), (32, 64, 0), (96, 32, 32), (64, 128, 0), (64, 256, 0), (128, 384, 0)])
def test_conv3x3_forward_and_data_gradient(torch_cuda, conv_impl, cin, cout, off):
    import ctypes as C
    import unet_ref as R
    from yapt_gb300 import _native as N
    from yapt_gb300.denoise import view
    torch = torch_cuda
    lib = N.load()
    rng = np.random.default_rng(cin + cout)
    n, h, w = 2, 12, 20
    stride_y = cout + off
    x = R.bf16(rng.normal(0, 1, (n, h, w, cin)))
    wt = R.bf16(rng.normal(0, 0.2, (cout, 3, 3, cin)))
    b = rng.normal(0, 0.1, cout).astype(np.float32)
    xd = dev_bf16(torch, x)
    wd = dev_bf16(torch, wt)
    bd = torch.from_numpy(b).cuda()
    yd = torch.zeros(n * h * w * stride_y, dtype=torch.bfloat16, device="cuda")
    rc = lib.yg_nn_conv3x3(C.byref(view(xd, cin, 0, cin)), C.c_void_p(wd.data_ptr()),
                           C.cast(C.c_void_p(bd.data_ptr()), C.POINTER(C.c_float)), C.byref(view(yd, stride_y, off, cout)),
                           None, 1, 0, n, h, w, stream(torch))
    assert rc == 0
    torch.cuda.synchronize()
    got = host(yd).reshape(n, h, w, stride_y)[..., off:]
    want = R.bf16(np.maximum(R.conv3x3(x, wt, b.astype(np.float64)), 0))
    np.testing.assert_allclose(got, want, rtol=2 ** -7, atol=1e-3)
    assert np.all(host(yd).reshape(n, h, w, stride_y)[..., :off] == 0)  # other channels untouched
    if cin % 32:
        return
    # data gradient through flipped weights, with a ReLU mask
    dy = R.bf16(rng.normal(0, 1, (n, h, w, cout)))
    mask = R.bf16(rng.normal(0, 1, (n, h, w, cin)))
    wf = torch.zeros_like(wd)
    assert lib.yg_nn_flip_weights(C.c_void_p(wd.data_ptr()), cout, cin, C.c_void_p(wf.data_ptr()), stream(torch)) == 0
    dyd, md = dev_bf16(torch, dy), dev_bf16(torch, mask)
    dxd = torch.zeros(n * h * w * cin, dtype=torch.bfloat16, device="cuda")
    rc = lib.yg_nn_conv3x3(C.byref(view(dyd, cout, 0, cout)), C.c_void_p(wf.data_ptr()), None,
                           C.byref(view(dxd, cin, 0, cin)), C.byref(view(md, cin, 0, cin)), 0, 0, n, h, w, stream(torch))
    assert rc == 0
    torch.cuda.synchronize()
    want = R.bf16(R.conv3x3_dgrad(dy, wt) * (mask > 0))
    np.testing.assert_allclose(host(dxd).reshape(n, h, w, cin), want, rtol=2 ** -7, atol=1e-3)


@pytest.mark.parametrize("cin,cout,off,masked", [(16, 32, 0, False), (32, 32, 0, True), (32, 64, 0, False), (64, 64, 0, True),
                                                  (96, 32, 32, False)])
def test_persistent_conv_matches_mma_sync_on_large_images(torch_cuda, cin, cout, off, masked):
    """Images of 65,536 pixels and more take the persistent TMA + tcgen05 kernel for these shapes
    (several tiles per CTA, double-buffered halo and accumulator). It must give what the mma.sync
    path gives to one BF16 rounding, with a ragged last tile (330 = 2 x 128 + 74 pixels), a ReLU
    mask and accumulation into the output, and no wait may run out."""
    import ctypes as C
    from yapt_gb300 import _native as N
    from yapt_gb300.denoise import view
    torch = torch_cuda
    lib = N.load()
    rng = np.random.default_rng(7 * cin + cout)
    n, h, w = 1, 200, 330
    stride_y = cout + off
    xd = dev_bf16(torch, rng.normal(0, 1, (n, h, w, cin)))
    wd = dev_bf16(torch, rng.normal(0, 0.2, (cout, 3, 3, cin)))
    bd = torch.from_numpy(rng.normal(0, 0.1, cout).astype(np.float32)).cuda()
    md = dev_bf16(torch, rng.normal(0, 1, (n, h, w, stride_y))) if masked else None
    y0 = dev_bf16(torch, rng.normal(0, 0.5, n * h * w * stride_y))
    outs = {}
    try:
        for impl in (0, 2):
            assert lib.yg_nn_set_conv_impl(impl) == 0
            yd = y0.clone()
            mv = C.byref(view(md, stride_y, off, cout)) if masked else None
            rc = lib.yg_nn_conv3x3(C.byref(view(xd, cin, 0, cin)), C.c_void_p(wd.data_ptr()),
                                   C.cast(C.c_void_p(bd.data_ptr()), C.POINTER(C.c_float)),
                                   C.byref(view(yd, stride_y, off, cout)), mv, 1, 1, n, h, w, stream(torch))
            assert rc == 0
            torch.cuda.synchronize()
            outs[impl] = host(yd).reshape(n, h, w, stride_y)
    finally:
        lib.yg_nn_set_conv_impl(0)
    t = C.c_uint32()
    assert lib.yg_nn_tc_timeouts(C.byref(t)) == 0 and t.value == 0, "tcgen05 waits ran out"
    a, b = outs[2], outs[0]
    assert np.array_equal(a[..., :off], host(y0).reshape(n, h, w, stride_y)[..., :off])  # other channels untouched
    np.testing.assert_allclose(a[..., off:], b[..., off:], rtol=2 ** -6, atol=2e-2)


@pytest.mark.parametrize("cin,cout", [(16, 32), (96, 32), (128, 256)])
def test_conv3x3_weight_gradient(torch_cuda, cin, cout):
    import ctypes as C
    import unet_ref as R
    from yapt_gb300 import _native as N
    from yapt_gb300.denoise import view
    torch = torch_cuda
    lib = N.load()
    rng = np.random.default_rng(7 + cin)
    n, h, w = 2, 40, 48
    x = R.bf16(rng.normal(0, 1, (n, h, w, cin)))
    dy = R.bf16(rng.normal(0, 1, (n, h, w, cout)))
    xd, dyd = dev_bf16(torch, x), dev_bf16(torch, dy)
    dw = torch.zeros(cout * 9 * cin, dtype=torch.float32, device="cuda")
    db = torch.zeros(cout, dtype=torch.float32, device="cuda")
    ws = torch.zeros(lib.yg_nn_wgrad_workspace(cin, cout, n, h, w) // 4 + 16, dtype=torch.float32, device="cuda")
    fp = lambda t: C.cast(C.c_void_p(t.data_ptr()), C.POINTER(C.c_float))  # noqa: E731
    rc = lib.yg_nn_conv3x3_wgrad(C.byref(view(xd, cin, 0, cin)), C.byref(view(dyd, cout, 0, cout)), fp(dw), fp(db),
                                 C.c_void_p(ws.data_ptr()), n, h, w, stream(torch))
    assert rc == 0
    torch.cuda.synchronize()
    want_w, want_b = R.conv3x3_wgrad(x, dy)
    got = dw.cpu().numpy().reshape(cout, 3, 3, cin)
    assert np.abs(got - want_w).max() <= 1e-3 * np.abs(want_w).max()
    np.testing.assert_allclose(db.cpu().numpy(), want_b, rtol=1e-4, atol=1e-3)


def test_pool_and_upsample_and_their_gradients(torch_cuda):
    import ctypes as C
    import unet_ref as R
    from yapt_gb300 import _native as N
    from yapt_gb300.denoise import view
    torch = torch_cuda
    lib = N.load()
    rng = np.random.default_rng(3)
    n, h, w, c = 2, 8, 12, 32
    x = R.bf16(rng.normal(0, 1, (n, h, w, c)))
    xd = dev_bf16(torch, x)
    pd = torch.zeros(n * h * w * c // 4, dtype=torch.bfloat16, device="cuda")
    assert lib.yg_nn_avgpool(C.byref(view(xd, c, 0, c)), C.byref(view(pd, c, 0, c)), n, h, w, stream(torch)) == 0
    ud = torch.zeros(n * h * w * c * 4, dtype=torch.bfloat16, device="cuda")
    assert lib.yg_nn_upsample(C.byref(view(xd, c, 0, c)), C.byref(view(ud, c, 0, c)), n, h, w, stream(torch)) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(host(pd).reshape(n, h // 2, w // 2, c), R.bf16(R.pool(x)), rtol=2 ** -7, atol=0)
    assert np.array_equal(host(ud).reshape(n, 2 * h, 2 * w, c), R.up(x))
    # backward: pool with skip add and mask, upsample with mask
    g = R.bf16(rng.normal(0, 1, (n, h // 2, w // 2, c)))
    add = R.bf16(rng.normal(0, 1, (n, h, w, c)))
    gd, ad, md = dev_bf16(torch, g), dev_bf16(torch, add), xd
    od = torch.zeros_like(xd)
    assert lib.yg_nn_avgpool_bwd(C.byref(view(gd, c, 0, c)), C.byref(view(ad, c, 0, c)), C.byref(view(md, c, 0, c)),
                                 C.byref(view(od, c, 0, c)), n, h, w, stream(torch)) == 0
    g2 = R.bf16(rng.normal(0, 1, (n, 2 * h, 2 * w, c)))
    g2d = dev_bf16(torch, g2)
    o2 = torch.zeros_like(xd)
    assert lib.yg_nn_upsample_bwd(C.byref(view(g2d, c, 0, c)), C.byref(view(md, c, 0, c)), C.byref(view(o2, c, 0, c)), n,
                                  h, w, stream(torch)) == 0
    torch.cuda.synchronize()
    np.testing.assert_allclose(host(od).reshape(n, h, w, c), R.bf16((R.pool_bwd(g) + add) * (x > 0)), rtol=2 ** -7, atol=0)
    np.testing.assert_allclose(host(o2).reshape(n, h, w, c), R.bf16(R.up_bwd(g2) * (x > 0)), rtol=2 ** -7, atol=0)


def test_unet_loss_and_gradients_match_the_oracle(torch_cuda, conv_impl):
    import unet_ref as R
    from yapt_gb300 import denoise as D
    torch = torch_cuda
    rng = np.random.default_rng(11)
    params = D.init_parameters(5)
    # non-zero biases so that every path of the network carries signal
    lay, _ = D.parameter_layout()
    for name, _, cout in D.LAYERS:
        b0 = lay[name][2]
        params[b0:b0 + cout] = rng.normal(0.02, 0.02, cout).astype(np.float32)
    n, h, w = 1, 16, 24
    x = np.zeros((n, h, w, 16))
    x[..., :10] = rng.uniform(0, 1, (n, h, w, 10))
    x = R.bf16(x)
    t = rng.uniform(0.05, 1.0, (n, h, w, 3))
    net = D.UNet(params)
    xd = dev_bf16(torch, x).reshape(-1)
    td = torch.from_numpy(t.astype(np.float32).reshape(-1)).cuda()
    loss = net.loss_and_gradients(xd, td, n, h, w)
    torch.cuda.synchronize()
    g = net.g.cpu().numpy().astype(np.float64)
    want_loss, want_g = R.loss_and_gradients(params, x, t.astype(np.float32).astype(np.float64))
    assert abs(loss - want_loss) <= 1e-2 * want_loss
    for name, _, _ in D.LAYERS + [("head", 0, 0)]:
        w0, nw, b0, nb = lay[name]
        a, b = g[w0:w0 + nw], want_g[w0:w0 + nw]
        cos = float(a @ b / (np.linalg.norm(a) * np.linalg.norm(b) + 1e-30))
        assert cos >= 0.999, (name, cos)
        assert abs(np.linalg.norm(a) / np.linalg.norm(b) - 1) < 0.02, name


def test_training_on_tracer_renders_beats_the_noisy_input(torch_cuda):
    from yapt_gb300 import configs
    from yapt_gb300 import denoise as D
    from yapt_gb300.runtime import Context
    torch = torch_cuda
    W = H = 64
    images, held = [], None
    with Context(0) as c:
        for seed in range(4):
            c.upload_scene(configs.box_scene(seed))
            xyz, alb, nrm, dep = D.render_features(c, W, H, 4)
            ref = D.render_reference(c, W, H, 256, spp_start=1000)
            item = (xyz, alb, nrm, dep, ref)
            if seed == 3:
                held = item
            else:
                images.append(item)
    net = D.UNet(seed=1)
    dev = [(D.to_device_input(net, *im[:4], depth_scale=4.0),
            torch.from_numpy(np.ascontiguousarray(im[4], np.float32).reshape(-1)).cuda(), H, W) for im in images]
    hist = D.train(net, dev, steps=600, batch=4, crop=48, lr=1e-3, seed=0)
    assert np.mean(hist[-20:]) < np.mean(hist[:20])
    xyz, alb, nrm, dep, ref = held
    noisy = xyz @ D.SRGB_FROM_XYZ.T
    den = D.denoise_image(net, D.to_device_input(net, xyz, alb, nrm, dep, depth_scale=4.0), H, W)
    r_noisy, r_den = D.relmse(noisy, ref), D.relmse(den, ref)
    assert np.all(np.isfinite(den))
    assert r_den < 0.7 * r_noisy, (r_den, r_noisy)  # three 64x64 training images: a sanity bound


def test_training_checkpoint_resumes_the_same_updates(torch_cuda, tmp_path):
    """A run restored from a checkpoint (FP32 weights, both Adam moments, step count) makes the
    same updates as the run that wrote it: six steps straight equal three, save, load, three."""
    from yapt_gb300 import denoise as D
    torch = torch_cuda
    n, h, w = 2, 32, 32
    rng = np.random.default_rng(3)
    x = dev_bf16(torch, rng.uniform(0, 1, (n * h * w * 16)))
    target = torch.from_numpy(rng.uniform(0, 1, n * h * w * 3).astype(np.float32)).cuda()

    def steps(net, k):
        for _ in range(k):
            net.loss_and_gradients(x, target, n, h, w)
            net.adam_step(lr=1e-3)

    a = D.UNet(seed=5)
    steps(a, 6)
    b = D.UNet(seed=5)
    steps(b, 3)
    path = str(tmp_path / "unet.npz")
    b.save_checkpoint(path)
    c = D.UNet.load_checkpoint(path)
    assert c.step_count == 3
    steps(c, 3)
    torch.cuda.synchronize()
    assert np.array_equal(a.parameters(), c.parameters())
