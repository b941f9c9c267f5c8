"""Generates tests/golden/golden.npz from the reference renderer itself.

Run in a checkout where the reference sources are available ($PETRICHOR_REF, or
a ``reference`` directory beside this repository): the reference's LibPetrichor is compiled unchanged by
oracle/ref/Makefile (with the project's stand-ins for its absent third-party
libraries) and driven by oracle/ref/harness.cpp through its public C++ API.
Each case stores the scene bytes it was rendered from, so the fixtures do not
depend on regenerating identical scenes elsewhere.

    python tests/golden/make_golden.py [--ref <reference checkout>]
"""
from __future__ import annotations

import argparse
import os
import sys

import numpy as np

ROOT = os.path.dirname(os.path.dirname(os.path.dirname(os.path.abspath(__file__))))
sys.path.insert(0, ROOT)

import oracle  # noqa: E402
from petrichor_gb300 import scene_io, synth  # noqa: E402

OUT = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden.npz")


def cases():
    """Scenes whose reference films are pinned (small, every material and integrator)."""
    return {
        "cornell_simple": synth.cornell(width=64, height=64, spp=16),
        "cornell_mixed_simple": synth.cornell(width=48, height=32, spp=8, mixed=True,
                                              aperture=0.05, env_texture=True),
        "cornell_mixed_pt": synth.cornell(width=48, height=32, spp=4, mixed=True, aperture=0.05,
                                          tile=7, integrator=1, max_bounces=6, env_texture=True),
        "cornell_lambert_pt": synth.cornell(width=40, height=40, spp=8, integrator=1, max_bounces=5),
        "spheres_pt": synth.spheres_grids(tri_budget=4000, width=48, height=27, spp=2,
                                          max_bounces=8, env_width=64, env_height=32),
        "textured_pt": synth.textured_spheres(integrator=1),
        "textured_simple": synth.textured_spheres(seed=6, integrator=0, spp=3),
        "uniform_lambert_simple": synth.uniform_lambert(
            synth.cornell(width=40, height=32, spp=8, mixed=True, env_texture=True)),
        "uniform_lambert_pt": synth.uniform_lambert(
            synth.cornell(width=40, height=40, spp=8, integrator=1, max_bounces=5), stride=1),
    }


def aov_cases():
    """Scenes whose AOV passes (UV, denoising albedo, denoising normal) are pinned, with
    their numSppForDenoising."""
    return {
        "aov_spheres": (synth.spheres_grids(tri_budget=4000, width=48, height=27, spp=2,
                                            max_bounces=8, env_width=64, env_height=32), 3),
        "aov_cornell_mixed": (synth.cornell(width=40, height=24, spp=3, mixed=True, aperture=0.05,
                                            tile=7, max_bounces=5, env_texture=True), 2),
        "aov_textured": (synth.textured_spheres(seed=7), 3),
    }


def main():
    ap = argparse.ArgumentParser()
    ap.add_argument("--ref", default=None,
                    help="reference checkout (default: $PETRICHOR_REF, else ../reference)")
    args = ap.parse_args()
    args.ref = args.ref or oracle.reference_root() or "(not found)"
    if oracle.build_reference(args.ref) is None:
        raise SystemExit(f"reference sources not found under {args.ref}")
    work = os.path.join(ROOT, "oracle", "_ref", "work")
    out = {}
    for name, sc in cases().items():
        out[f"{name}/scene"] = np.frombuffer(scene_io.scene_bytes(sc), np.uint8)
        film = np.frombuffer(oracle.run_reference("film", sc, work), np.float32)
        out[f"{name}/film"] = film.reshape(sc.settings.height, sc.settings.width, 3)
        print(name, "film mean", float(film.mean()))
    # BVH of the triangle-soup case and of a scene of equal sort keys and signed zeros;
    # primary hits and environment samples of the triangle-soup case
    bvh_scenes = {"spheres_pt": cases()["spheres_pt"], "bvh_ties": synth.bvh_ties()}
    for name, sc in bvh_scenes.items():
        if name not in cases():
            out[f"{name}/scene"] = np.frombuffer(scene_io.scene_bytes(sc), np.uint8)
        rb = oracle.run_reference("bvh", sc, work)
        nn, ni, depth = np.frombuffer(rb[:12], np.int32)
        arr = np.frombuffer(rb[12:12 + nn * 44], np.uint8).reshape(nn, 44)
        out[f"{name}/bvh_bounds"] = arr[:, :24].copy().view(np.float32).reshape(nn, 6)
        out[f"{name}/bvh_ints"] = arr[:, 24:].copy().view(np.int32).reshape(nn, 5)
        out[f"{name}/bvh_ids"] = np.frombuffer(rb[12 + nn * 44:], np.int32).copy()
        out[f"{name}/bvh_depth"] = np.array([depth], np.int32)
    sc = cases()["spheres_pt"]
    n = sc.settings.width * sc.settings.height
    rh = oracle.run_reference("hits", sc, work, 7, 11)
    out["spheres_pt/hit_rays"] = np.frombuffer(rh[:n * 32], np.float32).reshape(n, 8)
    out["spheres_pt/hits"] = np.frombuffer(rh[n * 32:], np.int32).reshape(n, 2)
    out["spheres_pt/env"] = np.frombuffer(oracle.run_reference("env", sc, work, 256),
                                          np.float32).reshape(256, 8)
    for name, (sc, dspp) in aov_cases().items():
        out[f"{name}/scene"] = np.frombuffer(scene_io.scene_bytes(sc), np.uint8)
        out[f"{name}/denoising_spp"] = np.array([dspp], np.int32)
        aov = np.frombuffer(oracle.run_reference("aov", sc, work, dspp), np.float32)
        out[f"{name}/aov"] = aov.reshape(3, sc.settings.height, sc.settings.width, 3)
        print(name, "aov means", [float(a.mean()) for a in out[f"{name}/aov"]])
    np.savez_compressed(OUT, **out)
    print("wrote", OUT, os.path.getsize(OUT), "bytes")


if __name__ == "__main__":
    main()
