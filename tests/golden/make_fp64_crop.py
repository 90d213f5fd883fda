"""Writes the FP64 judging fixture of the NEE random-shapes workload.

The workload: the NEE integrator on the random-shapes scene (500 icospheres of 320
triangles on a 40 x 40 ground quad, 3 blackbody quad lights; configs.random_shapes_scene(0)),
1024 x 1024 image, depth 12, spectral range 380..780 nm. The fixture is the 128 x 128 centre
crop (pixels 448..575 in x and y) rendered by the CPU oracle in double precision with the
4096 sample indices 0..4095, as 16 batches of 256 indices. It holds the mean XYZ per pixel
and the variance of that mean estimated from the spread of the 16 batch means, so a test can
tell Monte Carlo noise from a disagreement.

GPU renders judged against it must use other sample indices (4096 and up), so that the two
estimates are independent and their expected squared difference is the sum of their
variances.

  python tests/golden/make_fp64_crop.py [--threads N]

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

OUT = os.path.join(HERE, "nee_random_shapes_crop128_fp64_4096spp.npz")
SPEC = dict(scene="random_shapes_scene(seed=0)", integrator="nee", width=1024, height=1024, crop=[448, 448, 128, 128],
            max_depth=12, lambda_nm=[380, 780], spp_start=0, spp=4096, batches=16, precision=64)


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--threads", type=int, default=os.cpu_count() or 1)
    a = ap.parse_args()
    import pyoracle
    from yapt_gb300 import configs
    sc = configs.random_shapes_scene(0)
    h = pyoracle.OracleSceneHandle(sc, pyoracle.own_luts())
    per = SPEC["spp"] // SPEC["batches"]
    means = []
    t0 = time.time()
    for b in range(SPEC["batches"]):
        p = pyoracle.render_params(SPEC["integrator"], SPEC["width"], SPEC["height"], spp_start=SPEC["spp_start"] + b * per,
                                   spp=per, max_depth=SPEC["max_depth"], lambda_range=SPEC["lambda_nm"], crop=SPEC["crop"])
        means.append(h.render(p, precision=64, threads=a.threads, records=False, film=True)["film"])
        print("batch %d/%d  %.0f s" % (b + 1, SPEC["batches"], time.time() - t0), flush=True)
    m = np.stack(means)  # (batches, 128, 128, 3)
    mean = m.mean(axis=0)
    var_of_mean = m.var(axis=0, ddof=1) / SPEC["batches"]
    np.savez_compressed(OUT, mean=mean.astype(np.float32), var_of_mean=var_of_mean.astype(np.float32),
                        spec=json.dumps(SPEC))
    print("wrote %s (mean Y %.6f, %.0f s)" % (OUT, mean[..., 1].mean(), time.time() - t0))


if __name__ == "__main__":
    main()
