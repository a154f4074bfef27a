"""Shared test set-up: import paths, the `gpu` marker, and small seeded clouds."""
import os
import sys

import numpy as np
import pytest

REPO = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
PKG_ROOT = os.path.join(REPO, "c-_serial_gb300")
ORACLE = os.path.join(REPO, "oracle")
GOLDEN = os.path.join(REPO, "tests", "golden")
for p in (PKG_ROOT, ORACLE, os.path.join(REPO, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


def has_gpu() -> bool:
    try:
        import torch
        return torch.cuda.is_available()
    except Exception:
        return False


def pytest_collection_modifyitems(config, items):
    if has_gpu():
        return
    skip = pytest.mark.skip(reason="no CUDA GPU in this environment")
    for item in items:
        if "gpu" in item.keywords:
            item.add_marker(skip)


_clouds = {}


def small_cloud(n_wall=40, n_layers=12, seed=7, **kw):
    """A seeded NACA 0012 cloud small enough for the oracle to run in seconds."""
    from qlskum import cloudgen
    key = (n_wall, n_layers, seed, tuple(sorted(kw.items())))
    if key not in _clouds:
        _clouds[key] = cloudgen.make_cloud(n_wall=n_wall, n_layers=n_layers, first_spacing=kw.pop("first_spacing", 1e-2),
                                           radius=kw.pop("radius", 5.0), seed=seed, **kw)
    return _clouds[key]


def golden_cloud(name):
    """A cloud stored as a golden fixture (tests/golden/<name>.npz)."""
    from qlskum.cloudgen import Cloud
    z = np.load(os.path.join(GOLDEN, name + ".npz"))
    return Cloud(z["x"], z["y"], z["left"], z["right"], z["flag_1"], z["flag_2"], z["min_dist"], z["nbhs"],
                 z["conn"])


@pytest.fixture(scope="session")
def oracle_mod():
    import qlskum_oracle
    qlskum_oracle.build()
    return qlskum_oracle
