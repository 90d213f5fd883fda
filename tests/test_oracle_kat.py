"""Known-answer and consistency checks of the oracle's BSDF lobes and of energy conservation.

The reference holds no golden vectors for its BSDF math, so the oracle (and through per-sample
parity, the CUDA path) is checked against facts that need no reference output:
  * dielectric Fresnel at normal incidence is ((eta - 1) / (eta + 1))^2;
  * every importance sampler draws directions with the density its pdf reports (chi-square of
    histograms over the sphere against the pdf integrated per cell, plus the rejected mass);
  * the estimator f |cos| / pdf over a lobe's own samples converges to the lobe's directional
    albedo computed by quadrature;
  * the full layered BSDF, sampled as the integrators sample it (a layer chosen by its
    probability, then that layer's sampler), draws directions with the mixture pdf that
    evaluateSurface reports;
  * the dielectric-reflection and sheen lobes are reciprocal, f(wo, wi) = f(wi, wo);
  * white furnace (WHITE_FURNACE_TEST, raytraceCommon.hlsl:27-28): a convex white object under a
    constant environment looks like the environment, exactly for a Lambertian surface and
    within the multiple-scattering compensation's accuracy for a white rough conductor
    (Turquin, multiScatter.hlsl). (A coated diffuse surface is not a furnace invariant of the
    layered model: light leaving the base is not reflected back by the coat.)
The lobe checks run oracle/kat/kat.cpp (built by `make -C oracle kat`)."""
import json
import os
import subprocess
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
KAT = os.path.join(ROOT, "oracle", "_build", "kat")


@pytest.fixture(scope="module")
def kat():
    subprocess.run(["make", "-s", "-C", os.path.join(ROOT, "oracle"), "kat"], check=True)

    def run(*args):
        out = subprocess.run([KAT] + [str(a) for a in args], check=True, capture_output=True, text=True,
                             env=dict(os.environ, YAPT_DATA_DIR=os.path.join(ROOT, "yapt_gb300", "data"))).stdout
        return [json.loads(line) for line in out.splitlines() if line.startswith("{")]

    return run


def test_dielectric_fresnel_at_normal_incidence(kat):
    rows = kat("fresnel")
    assert len(rows) == 7
    for r in rows:
        assert abs(r["got"] - r["want"]) <= 1e-6 * max(r["want"], 1e-3), r


# (lobe, eta, alpha_x, alpha_y, cos of the outgoing direction): conductor reflection (0),
# dielectric reflection (1), transmission (2), dielectric reflection + transmission (3), cosine
# hemisphere (4); isotropic and anisotropic, near-normal and grazing, eta above and below 1
LOBES = [
    (4, 1.5, 0.5, 0.5, 0.7),
    (0, 1.5, 0.3, 0.3, 0.7),
    (0, 1.5, 0.6, 0.2, 0.4),
    (0, 1.5, 1.0, 1.0, 0.9),
    (0, 1.5, 0.5, 0.5, 0.15),
    (1, 1.5, 0.05, 0.05, 0.3),
    (2, 1.5, 0.3, 0.3, 0.7),
    (2, 1.5, 0.6, 0.6, 0.5),
    (3, 1.5, 0.3, 0.3, 0.7),
    (3, 1.0 / 1.5, 0.4, 0.4, 0.5),
    (3, 1.33, 0.8, 0.3, 0.2),
    (3, 1.0 / 1.5, 0.7, 0.7, 0.15),
]


@pytest.mark.parametrize("case", LOBES, ids=lambda c: "lobe%d-eta%.2f-a%.2fx%.2f-cos%.2f" % c)
def test_sampled_directions_follow_the_pdf(kat, case):
    chi2 = pytest.importorskip("scipy.stats").chi2
    r = kat("lobe", *case, 200000, 7)[0]
    p = float(chi2.sf(r["chi2"], r["dof"]))
    # a false alarm at 1e-4 per case; a wrong Jacobian or sampling routine gives p ~ 0
    assert p > 1e-4, r
    assert r["pdf_integral"] <= 1.0 + 2e-3, r
    if case[0] in (2, 4):  # samplers that never reject: all the mass inside the domain
        assert abs(r["pdf_integral"] - 1.0) < 2e-3 and r["rejected"] == 0, r


ALBEDO = [
    (1, 1.5, 0.3, 0.3, 0.7),
    (1, 1.5, 0.8, 0.4, 0.3),
    (2, 1.5, 0.3, 0.3, 0.7),
    (2, 1.33, 0.6, 0.6, 0.4),
    (5, 0.8, 0.5, 0.5, 0.7),
    (5, 0.8, 0.9, 0.9, 0.3),
]


@pytest.mark.parametrize("case", ALBEDO, ids=lambda c: "lobe%d-eta%.2f-a%.2fx%.2f-cos%.2f" % c)
def test_importance_sampled_albedo_matches_quadrature(kat, case):
    r = kat("albedo", *case, 200000, 11)[0]
    assert abs(r["estimate"] - r["quadrature"]) < 5.0 * r["stderr"] + 2e-4 * r["quadrature"], r


# presets of oracle/kat/kat.cpp: 0 clear coat + sheen + 30 % metal over diffuse, 1 rough glass,
# 2 rough plastic, 3 anisotropic metal under a rough coat
@pytest.mark.parametrize("preset", [0, 1, 2, 3])
@pytest.mark.parametrize("cos_wo", [0.7, 0.3])
def test_layered_bsdf_sampling_matches_its_mixture_pdf(kat, preset, cos_wo):
    chi2 = pytest.importorskip("scipy.stats").chi2
    r = kat("layered", preset, cos_wo, 200000, 3, os.path.join(ROOT, "yapt_gb300", "data"))[0]
    p = float(chi2.sf(r["chi2"], r["dof"]))
    assert p > 1e-4 and r["deltas"] == 0, r
    assert r["pdf_integral"] <= 1.0 + 2e-3, r


@pytest.mark.parametrize("lobe", [1, 5])
def test_reflection_lobes_are_reciprocal(kat, lobe):
    r = kat("reciprocity", lobe, 20000, 5)[0]
    assert r["pairs"] > 15000 and r["worst_rel"] < 1e-4, r


def furnace_ratio(material, integrator, spp=32, size=24):
    """Mean Y of the pixels that see a white icosphere (radius 1, 4 units from a 60-degree
    camera) over the mean Y of the pixels that see only the constant environment."""
    sys.path.insert(0, os.path.join(ROOT, "oracle"))
    import pyoracle
    from yapt_gb300 import _native as N
    from yapt_gb300 import configs
    from yapt_gb300.runtime import Context
    from yapt_gb300.scene import SPECTRUM_POINTS, CameraDesc, Scene
    sc = Scene()
    mesh = sc.add_mesh(*configs.icosphere(4))
    m = dict(material)
    m["albedo_spectrum"] = sc.add_spectrum(np.ones(SPECTRUM_POINTS, np.float32))
    sc.add_instance(mesh, sc.add_material(**m))
    sc.env_texture = sc.add_texture(np.ones((8, 16, 4), np.float32))
    sc.camera = CameraDesc(eye=(0.0, 0.0, 4.0), target=(0.0, 0.0, 0.0), fovy=np.pi / 3, aspect=1.0)
    p = Context.params(integrator, size, size, spp=spp, max_depth=8, lambda_range=(380, 780), flags=N.YG_FLAG_NO_FILM,
                       env_scale=1.0)
    rec = pyoracle.OracleSceneHandle(sc, pyoracle.own_luts(), N.host_table("rgb_to_spd", (380, 780))).render(
        p, precision=32)["records"]
    y = rec[..., 6].mean(axis=0)
    u = (np.arange(size) + 0.5) / size * 2.0 - 1.0
    angle = np.degrees(np.arctan(np.hypot(u[None, :], u[:, None]) * np.tan(np.pi / 6)))
    # the sphere subtends 14.5 degrees; pixels near its rim are left out
    return float(y[angle < 12.0].mean() / y[angle > 17.0].mean())


@pytest.mark.parametrize("integrator", ["uni", "nee"])
def test_white_lambertian_sphere_vanishes_in_a_furnace(built, integrator):
    ratio = furnace_ratio(dict(albedo=(1, 1, 1), metalness=0.0, transparency=0.0, specular_amount=0.0, roughness=1.0),
                          integrator)
    # one bounce to the environment with weight albedo = 1; what is left is the spread of the
    # hero-wavelength estimate of Y between pixels (~0.2 % per pixel)
    assert abs(ratio - 1.0) < 2e-3, ratio


@pytest.mark.parametrize("roughness", [0.3, 1.0])
def test_white_rough_conductor_keeps_its_energy(built, roughness):
    ratio = furnace_ratio(dict(albedo=(1, 1, 1), specular=(1, 1, 1), metalness=1.0, transparency=0.0,
                               specular_amount=1.0, roughness=roughness), "uni")
    # single scattering alone loses more energy the rougher the surface; the compensation
    # restores all but about 1 % of it
    assert 0.975 < ratio < 1.01, ratio
