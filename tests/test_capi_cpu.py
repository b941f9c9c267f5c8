"""The C-ABI library on a host without a GPU: it builds, loads and exports every
declared symbol; host-only entry points work; device entry points fail cleanly."""
import ctypes
import glob
import math
import os
import re
import subprocess

import numpy as np
import pytest

import oracle
from conftest import ROOT, golden_scene
from petrichor_gb300 import capi, synth


def _declared():
    names = set()
    for h in glob.glob(os.path.join(ROOT, "include", "*.h")):
        text = re.sub(r"/\*.*?\*/", "", open(h).read(), flags=re.S)
        names |= set(re.findall(r"\b(pt_[a-z0-9_]+)\s*\(", text))
    return names


def test_library_exports_every_declared_symbol():
    lib = capi.load()
    declared = _declared()
    assert declared, "no declarations found"
    assert declared == set(capi.EXPORTED)
    out = subprocess.run(["nm", "-D", "--defined-only", capi._build.LIB], capture_output=True,
                         text=True, check=True).stdout
    exported = set(re.findall(r"\s(pt_[a-z0-9_]+)$", out, flags=re.M))
    assert declared <= exported
    for n in declared:
        getattr(lib, n)


def test_status_strings():
    lib = capi.load()
    assert lib.pt_abi_version() == 5
    assert lib.pt_status_string(0) == b"ok"
    assert b"budget" in lib.pt_status_string(-3)


def test_context_without_device_reports_no_device():
    try:
        import torch
        if torch.cuda.is_available():
            pytest.skip("a CUDA device is present")
    except ImportError:
        pass
    lib = capi.load()
    h = ctypes.c_void_p()
    rc = lib.pt_context_create(0, 0, ctypes.byref(h))
    assert rc == -10 and not h.value


def test_camera_init_matches_reference_arithmetic():
    pos = np.array([0.0, -4.8, 1.0], np.float32)
    d = np.array([0.3, 1.0, -0.2], np.float32)
    cam = capi.PtCamera()
    tgt = np.array([-0.35, 0.3, 0.6], np.float32)
    rc = capi.load().pt_camera_init(capi._fptr(pos), capi._fptr(d), np.float32(0.7), 0.0,
                                    capi._fptr(tgt), 0.05, ctypes.byref(cam))
    assert rc == 0
    f = d / np.float32(np.sqrt(np.float64(np.dot(d, d))))
    right = np.cross(f, np.array([0, 0, 1], np.float32))
    assert np.allclose(np.array(cam.forward), f, rtol=0, atol=1e-7)
    assert np.allclose(np.array(cam.right), right, atol=1e-7)
    assert cam.h_perf == np.float32(2.0 * math.tan(np.float32(0.5) * np.float32(0.7)))
    assert abs(cam.focus_dist - float(np.linalg.norm(tgt - pos))) < 1e-6


def test_camera_init_rejects_missing_lens():
    cam = capi.PtCamera()
    z = np.zeros(3, np.float32)
    d = np.array([1, 0, 0], np.float32)
    assert capi.load().pt_camera_init(capi._fptr(z), capi._fptr(d), 0.0, 0.0, None, 0.0,
                                      ctypes.byref(cam)) == -1


@pytest.mark.parametrize("threads", [1, 3, 0])
def test_product_bvh_matches_reference_tree(golden, threads):
    sc = golden_scene(golden, "spheres_pt")
    b, q, ids, h = capi.bvh_build(sc.positions, sc.indices, threads=threads)
    assert np.array_equal(b.view(np.uint32), golden["spheres_pt/bvh_bounds"].view(np.uint32))
    assert np.array_equal(q, golden["spheres_pt/bvh_ints"])
    assert np.array_equal(ids, golden["spheres_pt/bvh_ids"])


def test_product_bvh_matches_reference_tree_on_equal_keys_and_signed_zeros(golden):
    """Equal sort keys on every axis and node bounds at +0 and -0: the host build must
    leave std::sort's order and the reference's first-of-equal bound merges."""
    sc = golden_scene(golden, "bvh_ties")
    b, q, ids, h = capi.bvh_build(sc.positions, sc.indices, threads=4)
    assert np.array_equal(b.view(np.uint32), golden["bvh_ties/bvh_bounds"].view(np.uint32))
    assert np.array_equal(q, golden["bvh_ties/bvh_ints"])
    assert np.array_equal(ids, golden["bvh_ties/bvh_ids"])


def test_product_bvh_matches_oracle_on_large_parallel_build():
    sc = synth.spheres_grids(tri_budget=150_000, width=8, height=8, spp=1, env_width=8, env_height=4)
    ob, oq, oids, _ = oracle.OracleScene(sc).bvh()
    b, q, ids, h = capi.bvh_build(sc.positions, sc.indices, threads=8)
    assert np.array_equal(b.view(np.uint32), ob.view(np.uint32))
    assert np.array_equal(q, oq) and np.array_equal(ids, oids)
    assert h < 64


def test_bvh_edge_cases():
    # empty scene: one empty root leaf
    b, q, ids, h = capi.bvh_build(np.zeros((0, 3), np.float32), np.zeros((0, 3), np.int32))
    assert b.shape[0] == 1 and q[0, 4] == 1 and ids.size == 0
    # identical centroids: never split (zero-width centroid range)
    P = np.array([[0, 0, 0], [1, 0, 0], [0, 1, 0]], np.float32)
    I = np.zeros((9, 3), np.int32) + np.array([0, 1, 2], np.int32)
    b, q, ids, h = capi.bvh_build(P, I)
    assert b.shape[0] == 1 and q[0, 3] == 9 and q[0, 4] == 1
    # bad index rejected
    with pytest.raises(capi.PtError):
        capi.bvh_build(P, np.array([[0, 1, 5]], np.int32))


def test_tuning_calls_reject_missing_context():
    lib = capi.load()
    t = capi.PtTuning()
    assert lib.pt_set_tuning(None, ctypes.byref(t)) == -1
    assert lib.pt_get_tuning(None, ctypes.byref(t)) == -1
    assert lib.pt_autotune(None, 1, None, None, 0, ctypes.byref(t)) == -1
