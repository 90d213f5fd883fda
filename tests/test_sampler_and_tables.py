"""Sampler and table checks that need no GPU.

The reference's own Sobol generator matrices (SobolMatrices.h, committed as the
golden fixture tests/golden/sobol_matrices_dims0_255.u32) pin both the library's
and the oracle's derivation from the Joe-Kuo direction numbers.
"""
import os

import numpy as np

from yapt_gb300 import _native as N

GOLDEN = os.path.join(os.path.dirname(__file__), "golden", "sobol_matrices_dims0_255.u32")


def golden_matrices():
    return np.fromfile(GOLDEN, dtype="<u4")


def test_library_sobol_matches_reference_table(built):
    assert np.array_equal(N.host_table("sobol"), golden_matrices())


def test_oracle_sobol_matches_reference_table(built):
    import pyoracle
    assert np.array_equal(pyoracle.sobol_matrices(), golden_matrices())


def sobol_point(m, index, dim):
    v = 0
    i = dim * 32
    while index:
        if index & 1:
            v ^= int(m[i])
        index >>= 1
        i += 1
    return v


def test_sobol_first_points_known_answers():
    m = golden_matrices()
    # dimension 0 is the van der Corput sequence in base 2
    assert [sobol_point(m, i, 0) / 2 ** 32 for i in range(8)] == [0, 0.5, 0.25, 0.75, 0.125, 0.625, 0.375, 0.875]
    # every dimension is a (0,1)-sequence: the first 2^k points stratify [0,1) into 2^k cells
    for d in range(0, 256, 17):
        pts = np.array([sobol_point(m, i, d) for i in range(64)], dtype=np.uint64)
        assert len(np.unique(pts >> np.uint64(26))) == 64


def test_cie_table_sums_match_reference_constants(built):
    cie = N.host_table("cie").reshape(471, 4).astype(np.float64)
    y = cie[20:341, 1]
    d65 = cie[20:341, 3]
    # CIE_Y_SUM / CIE_D65_SUM for 380..700 nm (spectralConstants.h:19-26)
    assert abs(y.sum() - 106.7989583) < 1e-4
    assert abs(d65.sum() - 29988.647) < 1e-2


def ggx_albedo_brute_force(mu, r, n=400000, seed=1):
    """Directional albedo of GGX (height-correlated Smith, no Fresnel) by uniform
    hemisphere sampling: an independent estimate of the quadrature the LUT holds."""
    rng = np.random.default_rng(seed)
    a = r * r
    wo = np.array([np.sqrt(1 - mu * mu), mu, 0.0])
    y = rng.random(n)
    s = np.sqrt(1 - y * y)
    phi = 2 * np.pi * rng.random(n)
    wi = np.stack([s * np.cos(phi), y, s * np.sin(phi)], 1)
    h = wi + wo
    h /= np.linalg.norm(h, axis=1, keepdims=True)
    D = 1 / (np.pi * a * a * ((h[:, 0] ** 2 + h[:, 2] ** 2) / (a * a) + h[:, 1] ** 2) ** 2)

    def lam(d):
        return (np.sqrt(1 + a * a * (d[..., 0] ** 2 + d[..., 2] ** 2) / d[..., 1] ** 2) - 1) / 2

    G2 = 1 / (1 + lam(wi) + lam(wo[None, :]))
    return np.mean(D * G2 / (4 * wo[1] * wi[:, 1]) * wi[:, 1]) * 2 * np.pi


def test_ms_luts_are_physical(host_luts):
    ss = host_luts["ss"].reshape(32, 32)  # [roughness][cos theta]
    assert np.all((ss > 0) & (ss <= 1.0001))
    for (ri, ci) in [(31, 1), (31, 16), (31, 31), (15, 8), (15, 31)]:
        r, mu = ri / 31.0, ci / 31.0
        assert abs(ss[ri, ci] - ggx_albedo_brute_force(mu, r)) < 0.01
    for k in ("trans_denser", "trans_lighter"):
        t = host_luts[k]
        assert np.all((t >= 0) & (t <= 1.01))
    assert host_luts["ssms"].size == 16 ** 3 and host_luts["sheen"].size == 256
    for k in ("trans_denser", "trans_lighter"):
        t = host_luts[k]
        assert np.all((t >= 0) & (t <= 1.01))
    assert host_luts["ssms"].size == 16 ** 3 and host_luts["sheen"].size == 256


def test_rgb_to_spd_fit_reproduces_grey_and_primaries(built):
    lut = N.host_table("rgb_to_spd", (380, 700)).reshape(64, 64, 64, 3)  # [b][g][r]

    def spd(coef, lam):
        x = coef[0] * lam * lam + coef[1] * lam + coef[2]
        return 0.5 * x / np.sqrt(1 + x * x) + 0.5

    lam = np.linspace(0, 1, 33)
    # a grey value fits an (almost) flat spectrum at that level
    grey = spd(lut[32, 32, 32], lam)
    assert np.ptp(grey) < 0.02 and abs(grey.mean() - 32 / 63) < 0.02
    # primaries put their energy in the right band (lam = (nm - 380) / 320)
    red, green, blue = lut[0, 0, 63], lut[0, 63, 0], lut[63, 0, 0]
    assert spd(red, 0.95) > 0.9 and spd(red, 0.35) < 0.1
    assert spd(green, 0.5) > 0.9 and spd(green, 0.95) < 0.1
    assert spd(blue, 0.2) > 0.9 and spd(blue, 0.8) < 0.1
