"""The a-trous denoiser's oracle on the CPU (no GPU).

The oracle (oracle/oracle_atrous.inc) restates the reference's edge-stopping a-trous filter
(Source/Renderer/shaders/postprocess/prefilterFeatures.comp, denoise.comp, denoiseFeatures.hlsl,
mergeNewSamples.comp) in FP32 in the device kernels' order. Here it is checked against an
independent float64 numpy restatement written from the same shader files, with the
reference's half-precision feature packing done by numpy's float16 (IEEE round to nearest
even, as HLSL f32tof16), and against properties of the filter: a flat image stays flat, the
feature packing round-trips, misses pass through, passes=0 returns the merged colour.
"""
import numpy as np
import pytest

from yapt_gb300 import configs

G3 = np.array([3 / 8, 1 / 4, 1 / 16])
G33 = np.array([[1 / 16, 1 / 8, 1 / 16], [1 / 8, 1 / 4, 1 / 8], [1 / 16, 1 / 8, 1 / 16]])
G33V = np.array([1 / 4, 1 / 8, 1 / 16])
DEFAULTS = dict(depth_sigma_scale=0.02, normal_sigma=0.06, material_sigma=0.05, color_sigma=3.0,
                feature_variance_scale=1.0, prefilter=1, passes=5)


@pytest.fixture(scope="module")
def oracle(built):
    import pyoracle
    return pyoracle


def params(**kw):
    from yapt_gb300.runtime import atrous_params
    d = dict(DEFAULTS)
    d.update(kw)
    return atrous_params(**d)


def camera(w, h):
    sc = configs.box_scene(0, aspect=w / h)
    return sc.camera.struct()


def synthetic(w, h, seed, spp=8, miss_frac=0.1):
    """Film sums, odd sums and moment sums of `spp` samples per pixel drawn around a few
    flat regions (per-pixel noisy features, some pixels with misses)."""
    rng = np.random.default_rng(seed)
    reg = (np.arange(w)[None, :] * 3 // w + 3 * (np.arange(h)[:, None] * 2 // h)).astype(int)
    nreg = reg.max() + 1
    alb_r = rng.uniform(0.05, 0.9, (nreg, 3))
    nrm_r = rng.normal(size=(nreg, 3))
    nrm_r /= np.linalg.norm(nrm_r, axis=1, keepdims=True)
    mat_r = rng.uniform(0, 1, (nreg, 4))
    ior_r = rng.uniform(1.0, 2.0, nreg)
    dep_r = rng.uniform(1.0, 5.0, nreg)
    lum_r = rng.uniform(0.05, 2.0, nreg)
    film = np.zeros((h, w, 4), np.float32)
    odd = np.zeros((h, w, 4), np.float32)
    mom = np.zeros((4, h, w, 4), np.float32)
    for s in range(spp):
        hit = rng.uniform(size=(h, w)) > miss_frac
        a = (alb_r[reg] + rng.normal(0, 0.02, (h, w, 3))).astype(np.float32)
        n = nrm_r[reg] + rng.normal(0, 0.05, (h, w, 3))
        n = (n / np.linalg.norm(n, axis=-1, keepdims=True)).astype(np.float32)
        m = np.clip(mat_r[reg] + rng.normal(0, 0.02, (h, w, 4)), 0, 1).astype(np.float32)
        ior = (ior_r[reg] * 0.5).astype(np.float32)
        d = (dep_r[reg] * (1 + rng.normal(0, 0.01, (h, w)))).astype(np.float32)
        y = (lum_r[reg] * rng.exponential(1.0, (h, w))).astype(np.float32)
        xyz = np.stack([y * 0.9, y, y * 1.1, np.ones_like(y)], -1).astype(np.float32)
        film += xyz
        if s & 1:
            odd += xyz
        layers = [np.concatenate([a, (a * a).sum(-1, keepdims=True)], -1),
                  np.concatenate([n, np.ones((h, w, 1), np.float32)], -1),
                  m,
                  np.stack([ior, (m * m).sum(-1) + ior * ior, d, d * d], -1)]
        for l in range(4):
            mom[l] += np.where(hit[..., None], layers[l], 0).astype(np.float32)
    return film, odd, mom


# ------------------------------------------------------------------ numpy restatement (float64)
def features_from_moments(film, mom):
    n = film[..., 3:4].astype(np.float64)
    inv = np.where(n > 0, 1.0 / np.where(n > 0, n, 1), 0.0)
    m = [mom[l].astype(np.float64) * inv for l in range(4)]
    f = {}
    f["albedo"] = m[0][..., :3]
    f["varAlbedo"] = np.maximum(m[0][..., 3] - (f["albedo"] ** 2).sum(-1), 0)
    f["normal"] = m[1][..., :3]
    cov = m[1][..., 3]
    f["mat"] = m[2]
    f["ior"] = m[3][..., 0]
    f["varMaterial"] = np.maximum(m[3][..., 1] - (m[2] ** 2).sum(-1) - f["ior"] ** 2, 0)
    safe = np.where(cov > 0, cov, 1)
    f["depth"] = np.where(cov > 0, m[3][..., 2] / safe, 0)
    f["varDepth"] = np.where(cov > 0, np.maximum(m[3][..., 3] / safe - f["depth"] ** 2, 0), 0)
    return f


def vnw(d2, sigma, var, k):
    return np.exp(-d2 / (sigma * sigma + k * var + 1e-8))


def feature_weight(c, s, P, k):
    nv = lambda f: np.clip(1 - np.linalg.norm(f["normal"], axis=-1), 0, 1)  # noqa: E731
    wn = vnw(((c["normal"] - s["normal"]) ** 2).sum(-1), P["normal_sigma"], nv(c) + nv(s), k)
    wa = vnw(((c["albedo"] - s["albedo"]) ** 2).sum(-1), P["material_sigma"], c["varAlbedo"] + s["varAlbedo"], k)
    wm = vnw(((c["mat"] - s["mat"]) ** 2).sum(-1) + (c["ior"] - s["ior"]) ** 2, P["material_sigma"],
             c["varMaterial"] + s["varMaterial"], k)
    return wn * wa * wm


def shifted(f, dx, dy):
    """f at (x + dx, y + dy) for every pixel, and the in-bounds mask."""
    h, w = next(iter(f.values())).shape[:2]
    ys, xs = np.mgrid[0:h, 0:w]
    sx, sy = xs + dx, ys + dy
    ok = (sx >= 0) & (sx < w) & (sy >= 0) & (sy < h)
    sxc, syc = np.clip(sx, 0, w - 1), np.clip(sy, 0, h - 1)
    return {k: v[syc, sxc] for k, v in f.items()}, ok


def prefilter(f, P):
    k = P["feature_variance_scale"]
    acc = {n: 0.0 for n in ("albedo", "normal", "mat", "ior", "w", "d", "dw", "va", "vm", "vd", "vw")}

    def rdw(c, s, kk):
        both = (c["depth"] > 0) & (s["depth"] > 0)
        d = c["depth"] - s["depth"]
        return np.where(both, vnw(d * d, c["depth"] * P["depth_sigma_scale"], c["varDepth"] + s["varDepth"], kk), 1.0)

    for dy in range(-2, 3):
        for dx in range(-2, 3):
            s, ok = shifted(f, dx, dy)
            w = np.where(ok, G3[abs(dx)] * G3[abs(dy)] * feature_weight(f, s, P, k) * rdw(f, s, k), 0)
            acc["albedo"] = acc["albedo"] + s["albedo"] * w[..., None]
            acc["normal"] = acc["normal"] + s["normal"] * w[..., None]
            acc["mat"] = acc["mat"] + s["mat"] * w[..., None]
            acc["ior"] = acc["ior"] + s["ior"] * w
            acc["w"] = acc["w"] + w
            hitw = np.where(s["depth"] > 0, w, 0)
            acc["d"] = acc["d"] + s["depth"] * hitw
            acc["dw"] = acc["dw"] + hitw
            if abs(dx) <= 1 and abs(dy) <= 1:
                wv = np.where(ok, G33V[abs(dx) + abs(dy)] * feature_weight(f, s, P, 0.0) * rdw(f, s, 0.0), 0)
                acc["va"] = acc["va"] + s["varAlbedo"] * wv
                acc["vm"] = acc["vm"] + s["varMaterial"] * wv
                acc["vd"] = acc["vd"] + np.where(s["depth"] > 0, s["varDepth"], f["varDepth"]) * wv
                acc["vw"] = acc["vw"] + wv
    inv = 1 / np.maximum(acc["w"], 1e-6)
    r = dict(f)
    r["albedo"] = acc["albedo"] * inv[..., None]
    r["normal"] = acc["normal"] * inv[..., None]
    r["mat"] = acc["mat"] * inv[..., None]
    r["ior"] = acc["ior"] * inv
    r["depth"] = np.where((f["depth"] > 0) & (acc["dw"] > 0), acc["d"] / np.where(acc["dw"] > 0, acc["dw"], 1), f["depth"])
    iv = 1 / np.maximum(acc["vw"], 1e-6)
    r["varAlbedo"], r["varMaterial"], r["varDepth"] = acc["va"] * iv, acc["vm"] * iv, acc["vd"] * iv
    return r


def half(x):
    return np.asarray(x, np.float32).astype(np.float16).astype(np.float64)


def pack_roundtrip(f):
    """writeDenoiseFeatures then readDenoiseFeatures: halves except depth (a full float)."""
    d = f["depth"].astype(np.float32).astype(np.float64)
    rel = np.where(d > 0, np.minimum(f["varDepth"] / np.where(d > 0, d * d, 1), 65000), 0)
    g = dict(albedo=half(f["albedo"]), normal=half(f["normal"]), mat=half(f["mat"]), ior=half(f["ior"]), depth=d,
             varAlbedo=half(np.minimum(f["varAlbedo"], 65000)), varMaterial=half(np.minimum(f["varMaterial"], 65000)))
    g["varDepth"] = half(rel) * d * d
    return g


def merged(film, odd):
    n, no = film[..., 3].astype(np.float64), odd[..., 3].astype(np.float64)
    ne = n - no
    both = (ne > 0) & (no > 0)
    ev = (film[..., :3] - odd[..., :3]) / np.where(both, ne, 1)[..., None]
    ov = odd[..., :3] / np.where(both, no, 1)[..., None]
    col = np.where(both[..., None], (ev + ov) / 2, film[..., :3] / np.where(n > 0, n, 1)[..., None])
    var = np.where(both, (np.log1p(ev[..., 1]) - np.log1p(ov[..., 1])) ** 2 / 2, 0)
    return col, var


def world_pos(cam, depth):
    h, w = depth.shape
    U = np.array(cam.uv_to_view, np.float64).reshape(4, 4)
    V = np.array(cam.view_to_world, np.float64).reshape(4, 4)
    ys, xs = np.mgrid[0:h, 0:w]
    uv = np.stack([(xs + 0.5) / w, (ys + 0.5) / h, np.zeros_like(xs, float), np.ones_like(xs, float)], -1)
    p = uv @ U.T
    p = p / p[..., 3:4]
    pos = p[..., :3] * (depth / np.maximum(np.abs(p[..., 2]), 1e-8))[..., None]
    return (np.concatenate([pos, np.ones_like(depth)[..., None]], -1) @ V.T)[..., :3]


def atrous_numpy(film, odd, mom, cam, P):
    f = features_from_moments(film, mom)
    if P["prefilter"]:
        f = prefilter(f, P)
    f = pack_roundtrip(f)
    col, var = merged(film, odd)
    pos = world_pos(cam, f["depth"])
    f["pos"] = pos
    k = P["feature_variance_scale"]
    for p in range(P["passes"]):
        vs, vw = 0.0, 0.0
        for dy in range(-1, 2):
            for dx in range(-1, 2):
                s, ok = shifted(dict(v=var), dx, dy)
                vs = vs + np.where(ok, s["v"] * G33[dx + 1, dy + 1], 0)
                vw = vw + np.where(ok, G33[dx + 1, dy + 1], 0)
        std = np.sqrt(np.maximum(vs / np.maximum(vw, 1e-6), 1e-6))
        sc_, sv_, sw_ = 0.0, 0.0, 0.0
        step = 1 << p
        nl = np.linalg.norm(f["normal"], axis=-1)
        nn = f["normal"] / np.where(nl > 1e-3, nl, 1)[..., None]
        for dy in range(-2, 3):
            for dx in range(-2, 3):
                s, ok = shifted(dict(f, col=col, var=var), dx * step, dy * step)
                dist = np.where(nl > 1e-3, (nn * (s["pos"] - f["pos"])).sum(-1), f["depth"] - s["depth"])
                wd = np.where(s["depth"] > 0, vnw(dist * dist, f["depth"] * P["depth_sigma_scale"],
                                                  f["varDepth"] + s["varDepth"], k), 1.0)
                wc = np.exp(-np.abs(s["col"][..., 1] - col[..., 1]) / (P["color_sigma"] * std + 1e-6))
                w = np.where(ok, G3[abs(dx)] * G3[abs(dy)] * wd * feature_weight(f, s, P, k) * wc, 0)
                sc_ = sc_ + s["col"] * w[..., None]
                sv_ = sv_ + w * w * s["var"]
                sw_ = sw_ + w
        inv = 1 / np.maximum(sw_, 1e-6)
        keep = f["depth"] <= 0
        col = np.where(keep[..., None], col, sc_ * inv[..., None])
        var = np.where(keep, 0, sv_ * inv * inv)
    return col, var


# ------------------------------------------------------------------ tests
@pytest.mark.parametrize("prefilter", [0, 1])
def test_oracle_matches_the_numpy_restatement(oracle, prefilter):
    h, w = 24, 36
    film, odd, mom = synthetic(w, h, seed=3 + prefilter)
    cam = camera(w, h)
    P = dict(DEFAULTS, prefilter=prefilter)
    out, var, _ = oracle.atrous(film, odd, mom, cam, params(**P))
    ref_c, ref_v = atrous_numpy(film, odd, mom, cam, P)
    np.testing.assert_allclose(out[..., :3], ref_c, rtol=2e-4, atol=1e-6)
    np.testing.assert_allclose(var, ref_v, rtol=2e-3, atol=1e-7)


def test_packed_features_are_ieee_halves_of_the_resolved_moments(oracle):
    h, w = 16, 20
    film, odd, mom = synthetic(w, h, seed=11, miss_frac=0.3)
    # stretch some values into the half subnormal range and past the largest half
    mom[0, 0, :5, 0] *= np.float32(1e-6)
    mom[0, 1, :5, 1] = np.float32(7e5)
    _, _, feat = oracle.atrous(film, odd, mom, camera(w, h), params(prefilter=0, passes=0))
    f = features_from_moments(film, mom)
    n = film[..., 3:4]
    inv = np.where(n > 0, np.float32(1) / np.where(n > 0, n, 1), 0).astype(np.float32)
    m0 = (mom[0] * inv).astype(np.float32)
    lo = lambda v: (v & 0xFFFF).astype(np.uint16).view(np.float16)  # noqa: E731
    hi = lambda v: (v >> 16).astype(np.uint16).view(np.float16)  # noqa: E731
    assert np.array_equal(lo(feat[0, ..., 0]), m0[..., 0].astype(np.float16))
    with np.errstate(over="ignore"):  # 7e5 rounds to +inf in half precision, as intended
        assert np.array_equal(hi(feat[0, ..., 0]), m0[..., 1].astype(np.float16))
    assert np.array_equal(lo(feat[0, ..., 1]), m0[..., 2].astype(np.float16))
    assert np.isinf(hi(feat[0, 1, :5, 0]).astype(np.float32)).all()
    depth = feat[1, ..., 0].view(np.float32)
    np.testing.assert_allclose(depth, f["depth"], rtol=1e-6)
    assert np.all((depth == 0) == (mom[1, ..., 3] == 0))


def test_flat_image_stays_flat_and_misses_pass_through(oracle):
    h, w = 20, 24
    film, odd, mom = synthetic(w, h, seed=5, miss_frac=0.0)
    # one region, constant colour, identical features everywhere
    film[..., :3] = np.float32(0.5) * film[..., 3:4]
    odd[..., :3] = np.float32(0.5) * odd[..., 3:4]
    for l in range(4):
        mom[l] = mom[l, :1, :1] / film[:1, :1, 3:4] * film[..., 3:4]
    mom[:, 3, 4] = 0  # a pixel without hits
    film[3, 4, :3] = [2.0 * film[3, 4, 3], 0.0, 0.0]
    out, var, _ = oracle.atrous(film, odd, mom, camera(w, h), params())
    assert np.allclose(np.delete(out.reshape(-1, 4), 3 * w + 4, 0)[:, 1], 0.5, rtol=1e-5)
    assert np.array_equal(out[3, 4, :3], np.float32([2.0, 0.0, 0.0]))
    assert var[3, 4] == 0.0


def test_zero_passes_return_the_merged_colour(oracle):
    h, w = 12, 10
    film, odd, mom = synthetic(w, h, seed=9)
    out, var, _ = oracle.atrous(film, odd, mom, camera(w, h), params(passes=0))
    col, v = merged(film, odd)
    np.testing.assert_allclose(out[..., :3], col, rtol=1e-6)
    np.testing.assert_allclose(var, v, rtol=1e-4, atol=1e-9)


def test_library_exports_the_atrous_entry_points(built):
    from yapt_gb300 import _native as N
    lib = N.load()
    for name in ("yg_atrous_default_params", "yg_atrous_denoise", "yg_atrous_read", "yg_atrous_run"):
        assert hasattr(lib, name)
    p = params()
    assert (p.prefilter, p.passes) == (1, 5)
    assert abs(p.color_sigma - 3.0) < 1e-7 and abs(p.depth_sigma_scale - 0.02) < 1e-7
