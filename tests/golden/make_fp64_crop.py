"""Writes the FP64 judging fixtures of the benchmark workloads.

Each fixture is a 128 x 128 centre crop of a workload rendered by the CPU oracle in double
precision with the 4096 sample indices 0..4095, as 16 batches of 256 indices. It holds the
mean XYZ per pixel and the variance of that mean estimated from the spread of the 16 batch
means, so a test can tell Monte Carlo noise from a disagreement.

  nee_random_shapes  the NEE integrator on the random-shapes scene (500 icospheres of 320
                     triangles on a 40 x 40 ground quad, 3 blackbody quad lights;
                     configs.random_shapes_scene(0)), 1024 x 1024, depth 12, pixels 448..575
  bdpt_caustic_box   the BDPT integrator on the caustic box (configs.caustic_box_scene(0),
                     ~196k triangles), 512 x 512, camera and light depth 10, pixels 192..319
  nee_caustic_box    the NEE integrator on the same caustic-box crop, depth 10 (BDPT and NEE
                     use different multiple-scattering models on rough dielectrics, as in the
                     reference, so each integrator is judged against its own converged image)

All at 380..780 nm. GPU renders judged against a fixture must use other sample indices (4096
and up), so that the two estimates are independent and their expected squared difference is
the sum of their variances.

  python tests/golden/make_fp64_crop.py [--threads N] [--only NAME]

TEST INFRASTRUCTURE: runs the oracle only (no GPU, no GPU library).
"""
import argparse
import json
import os
import sys
import time

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "oracle"))

FIXTURES = {
    "nee_random_shapes": dict(scene="random_shapes_scene(seed=0)", integrator="nee", width=1024, height=1024,
                              crop=[448, 448, 128, 128], max_depth=12, lambda_nm=[380, 780], spp_start=0, spp=4096,
                              batches=16, precision=64),
    "bdpt_caustic_box": dict(scene="caustic_box_scene(seed=0)", integrator="bdpt", width=512, height=512,
                             crop=[192, 192, 128, 128], max_depth=10, light_vertices=10, lambda_nm=[380, 780],
                             spp_start=0, spp=4096, batches=16, precision=64),
    "nee_caustic_box": dict(scene="caustic_box_scene(seed=0)", integrator="nee", width=512, height=512,
                            crop=[192, 192, 128, 128], max_depth=10, lambda_nm=[380, 780], spp_start=0, spp=4096,
                            batches=16, precision=64),
}


def path(name):
    return os.path.join(HERE, "%s_crop128_fp64_4096spp.npz" % name)


def make(name, threads):
    import pyoracle
    from yapt_gb300 import configs
    spec = FIXTURES[name]
    sc = eval("configs." + spec["scene"], {"configs": configs})
    h = pyoracle.OracleSceneHandle(sc, pyoracle.own_luts())
    per = spec["spp"] // spec["batches"]
    means = []
    t0 = time.time()
    for b in range(spec["batches"]):
        p = pyoracle.render_params(spec["integrator"], spec["width"], spec["height"], spp_start=spec["spp_start"] + b * per,
                                   spp=per, max_depth=spec["max_depth"], lambda_range=spec["lambda_nm"], crop=spec["crop"],
                                   light_vertices=spec.get("light_vertices", 0))
        h.ensure_rgb_table(p)
        means.append(h.render(p, precision=64, threads=threads, records=False, film=True)["film"])
        print("%s batch %d/%d  %.0f s" % (name, b + 1, spec["batches"], time.time() - t0), flush=True)
    m = np.stack(means)  # (batches, 128, 128, 3)
    mean = m.mean(axis=0)
    var_of_mean = m.var(axis=0, ddof=1) / spec["batches"]
    np.savez_compressed(path(name), mean=mean.astype(np.float32), var_of_mean=var_of_mean.astype(np.float32),
                        spec=json.dumps(spec))
    print("wrote %s (mean Y %.6f, %.0f s)" % (path(name), mean[..., 1].mean(), time.time() - t0))


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    ap.add_argument("--only", choices=sorted(FIXTURES))
    a = ap.parse_args()
    for name in ([a.only] if a.only else sorted(FIXTURES)):
        make(name, a.threads)


if __name__ == "__main__":
    main()
