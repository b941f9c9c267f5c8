import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

GOLDEN = os.path.join(ROOT, "tests", "golden", "golden.npz")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300)")


@pytest.fixture(scope="session")
def golden():
    with np.load(GOLDEN) as z:
        return {k: z[k] for k in z.files}


def golden_scene(golden, name):
    from petrichor_gb300 import scene_io
    return scene_io.read_scene_bytes(golden[f"{name}/scene"].tobytes())


GOLDEN_CASES = ["cornell_simple", "cornell_mixed_simple", "cornell_mixed_pt", "cornell_lambert_pt",
                "spheres_pt", "textured_pt", "textured_simple", "uniform_lambert_simple",
                "uniform_lambert_pt"]
AOV_CASES = ["aov_spheres", "aov_cornell_mixed", "aov_textured"]  # UV, denoising albedo, normal


@pytest.fixture(scope="session")
def gpu_ctx():
    from petrichor_gb300 import capi
    ctx = capi.Context()
    yield ctx
    ctx.close()
