"""Generates the committed FP64-oracle fixtures under tests/golden/.

The reference (merian's Vulkan/Slang `pt`) cannot run here, so its estimator is pinned by the
FP64 CPU oracle (oracle/oracle.cpp, a restatement of render_pt.slang): each fixture holds, for a
seeded subset of pixels, the oracle's per-pixel mean radiance over many BSDF-only samples and the
per-sample variance, the output's `a` channel (mean squared luminance) with the variance of its
samples, plus a hash of the scene arrays it was computed on. Scenes and cameras come from the
oracle library (the seeded generators compiled into it and its own camera basis), so making a
fixture never loads the CUDA library; the GPU tests re-hash the scene the package generates.

    python tests/golden/make_golden.py [--quick]
"""
from __future__ import annotations

import argparse
import hashlib
import sys
import time
from pathlib import Path

import numpy as np

ROOT = Path(__file__).resolve().parents[2]
sys.path.insert(0, str(ROOT))

from merian_gb300 import scene as S  # noqa: E402
from oracle import binding as O  # noqa: E402

HERE = Path(__file__).resolve().parent


def scene_hash(sc) -> str:
    h = hashlib.sha256()
    for a in (sc.vertices, sc.indices, sc.geometries, sc.materials):
        h.update(np.ascontiguousarray(a).tobytes())
    if sc.env is not None:
        h.update(np.ascontiguousarray(sc.env).tobytes())
    return h.hexdigest()


# name -> (scene factory, camera, width, height, max_path_length, n_pixels, spp)
def cases():
    gen = O.generator()
    return {
        "cornell": dict(
            scene=lambda: S.cornell(S.BASE_SEED, lib=gen),
            camera=lambda: O.workload_camera("cornell-256-16spp"),
            width=256, height=256, max_path_length=5, n_pixels=1024, spp=65536),
        "soup_small": dict(
            scene=lambda: S.soup(S.BASE_SEED, 200_000, 256, (256, 128), lib=gen),
            camera=lambda: O.look_at((0.5, 0.5, -1.2), (0.5, 0.5, 0.5), (0, 1, 0), 45.0, 16 / 9),
            width=320, height=180, max_path_length=8, n_pixels=512, spp=16384),
        # the headline configuration: the benchmarked 1M-triangle soup with its 2048x1024
        # environment, seen by the 1080p camera
        "soup_1m": dict(
            scene=lambda: S.workload_scene("soup-1m-1080p-64spp", lib=gen),
            camera=lambda: O.workload_camera("soup-1m-1080p-64spp"),
            width=1920, height=1080, max_path_length=8, n_pixels=1024, spp=65536),
        # the same, 64 pixels deep enough (2^22 spp) that the fixture's own noise stays well
        # below 1 % relative RMSE: the pin for the relative-RMSE figure the benchmark reports
        "soup_1m_deep": dict(
            scene=lambda: S.workload_scene("soup-1m-1080p-64spp", lib=gen),
            camera=lambda: O.workload_camera("soup-1m-1080p-64spp"),
            width=1920, height=1080, max_path_length=8, n_pixels=64, spp=1 << 22),
    }


def make(name: str, c: dict, spp_scale: float = 1.0) -> Path:
    sc = c["scene"]()
    cam = c["camera"]()
    w, h = c["width"], c["height"]
    rng = np.random.default_rng(0x1234567)
    pixels = np.sort(rng.choice(w * h, size=c["n_pixels"], replace=False)).astype(np.uint32)
    spp = max(64, int(c["spp"] * spp_scale))
    params, keep = S.render_params(w, h, spp, c["max_path_length"], pixels=pixels)
    osc = O.OracleScene(sc)
    t0 = time.time()
    rgba, sq, rays, lum4 = osc.render(cam, params, fp64=True, lum4=True)
    dt = time.time() - t0
    mean = rgba[:, :3]
    var = np.maximum(sq - mean * mean, 0.0)
    var_lum2 = np.maximum(lum4 - rgba[:, 3] ** 2, 0.0)
    out = HERE / f"{name}.npz"
    np.savez_compressed(out, pixels=pixels, mean=mean, var=var, lum2=rgba[:, 3],
                        var_lum2=var_lum2, spp=spp,
                        width=w, height=h, max_path_length=c["max_path_length"],
                        scene_hash=scene_hash(sc), oracle_seconds=dt, rays=rays)
    print(f"{name}: {len(pixels)} px x {spp} spp in {dt:.1f} s -> {out}")
    return out


if __name__ == "__main__":
    ap = argparse.ArgumentParser()
    ap.add_argument("--quick", action="store_true", help="1/64 of the samples (smoke only)")
    ap.add_argument("--only", default=None)
    args = ap.parse_args()
    for name, c in cases().items():
        if args.only and name != args.only:
            continue
        make(name, c, 1 / 64 if args.quick else 1.0)
