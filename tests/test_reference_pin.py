"""The oracle pinned to the reference's own shader code (no GPU).

oracle/ref_build.py compiles the reference's HLSL shader math (random.hlsl,
randomSampler.hlsl, spectralDistribution.hlsl, ggx.hlsl, fresnel.hlsl, miscBrdf.hlsl,
bsdfSample.hlsl, multiScatter.hlsl, materialLayers.hlsl, materialSample.hlsl and the
subsurface functions of subsurface.hlsl) as C++
through oracle/hlsl_shim.h into oracle/_ref/refcheck, once as the unidirectional
integrators compile it and once with RECIPROCAL_MULTISCATTER as the bidirectional one does,
and runs it beside the oracle's restatement on the same seeded inputs. The sampler is
compared bit for bit; every other function within 1e-4 relative, the per-sample parity
tolerance. Skipped where the reference's shader sources are not present.
"""
import json
import os
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, os.path.join(ROOT, "oracle"))

import ref_build  # noqa: E402

# the functions the oracle restates, by the reference's names: none may drop out of the check
EXPECTED = [
    "hash(a,b)", "owenScrambleBase2Fast", "uintToFloat01", "RandomSampler (texel offset, 40 dimensions)",
    "getSpectralSampleLambdas", "sigmoid", "setFromRGB", "setFromRGBUnbounded", "setFromRGBUnboundedNoIlluminant",
    "ToXYZ", "applyRussianRoulette", "smithLambdaGGX", "G1GGX", "G2GGX", "DGGX", "DVGGX",
    "sampleWMGGX (visible normals)", "getConductorRefractiveIndexAndExtinction", "fresnelDielectricConductor",
    "fresnelDielectricDielectric2", "DSheen", "GSheen", "evaluateEmissionProfile", "sampleConcentricDisk",
    "sampleGGXReflectionConductor", "pdfGGXReflectionConductor", "sampleGGXReflectionDielectric",
    "pdfGGXReflectionDielectric", "evaluateGGXReflectionDielectric", "pdfGGXTransmitted", "evaluateGGXTransmitted",
    "sampleDielectric", "pdfDielectric", "sampleDiffuseLambertian", "pdfDiffuseLambertian", "sampleSheen", "pdfSheen",
    "evaluateSheen", "getEnergyCompensationTurquin", "getEnergyCompensationKulla", "getEnergyRemainingAfterSpecular",
    "getEnergyRemainingAfterSheen", "getEnergyCompensationTranslucentTurquin", "getEnergyCompensationTranslucentKulla",
    "getAvgFresnel", "getMsTransmissionRatio", "getFmsDielectric", "getSheenDirectionalAlbedo",
    "getDirectionalAlbedoTranslucent", "getAverageAlbedoTranslucent",
    "calculateNormalizedMaterialLayerSamplingProbabilities", "getSampleDirectionOSForLayer",
    "evaluateSurface (weight)", "evaluateSurface (pdf)", "evaluateSurface (transmission type)",
    "burleyProfileArea", "burleySampleRadius", "burleyD", "pdfSubsurfaceExit", "getSubsurfaceEntryFactor",
    "sampleSubsurfaceExitLobe", "evaluateSubsurfaceExitLobe",
    "getSampleDirectionOSForLayer (RECIPROCAL_MULTISCATTER)", "evaluateSurface (RECIPROCAL_MULTISCATTER, weight)",
    "evaluateSurface (RECIPROCAL_MULTISCATTER, pdf)", "evaluateSurface (RECIPROCAL_MULTISCATTER, transmission type)",
]


@pytest.fixture(scope="module")
def report():
    if not os.path.isdir(ref_build.SHADERS):
        pytest.skip("the reference's shader sources are not present on this machine")
    assert ref_build.build()
    r = subprocess.run([ref_build.BIN, os.path.join(ROOT, "yapt_gb300", "data"), "30000"], stdout=subprocess.PIPE,
                       text=True, timeout=600)
    rep = json.loads(r.stdout)
    rep["rc"] = r.returncode
    return rep


def test_every_restated_function_is_compared(report):
    names = [c["name"] for c in report["checks"]]
    assert names == EXPECTED


@pytest.mark.parametrize("name", EXPECTED)
def test_oracle_matches_the_reference_shader_code(report, name):
    c = next(c for c in report["checks"] if c["name"] == name)
    assert c["n"] > 1000
    assert c["pass"], c
    if c["exact"]:
        assert c["within"] == 1.0, c


def test_the_comparison_reports_success(report):
    assert report["ok"] and report["rc"] == 0
