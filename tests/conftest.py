"""Shared fixtures: the package (loaded from its directory), the oracle and
the golden fixtures made from the reference's own code."""
from __future__ import annotations

import importlib.util
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
PKG_DIR = ROOT / "bachelorarbeit-mlem_gb300"
GOLDEN = ROOT / "tests" / "golden" / "reference_outputs.npz"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300 box)")


def load_pkg():
    if "mlem_gb300" in sys.modules:
        return sys.modules["mlem_gb300"]
    spec = importlib.util.spec_from_file_location("mlem_gb300", PKG_DIR / "__init__.py",
                                                  submodule_search_locations=[str(PKG_DIR)])
    m = importlib.util.module_from_spec(spec)
    sys.modules["mlem_gb300"] = m
    spec.loader.exec_module(m)
    return m


def build_pkg():
    spec = importlib.util.spec_from_file_location("mlem_gb300_build", PKG_DIR / "build.py")
    b = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(b)
    return b.build()


@pytest.fixture(scope="session")
def pkg():
    build_pkg()
    return load_pkg()


@pytest.fixture(scope="session")
def O():
    from oracle import oracle
    return oracle


@pytest.fixture(scope="session")
def golden():
    return np.load(GOLDEN)


def golden_cases(z):
    return sorted({k.split("/")[0] for k in z.files if k.split("/")[0] != "csr4"})


def golden_csr(z, name):
    return z[f"{name}/rowptr"], z[f"{name}/col"], z[f"{name}/val"], int(z[f"{name}/cols"])


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    return torch


def problem(pkg, O, name, n_shapes=5, total=1e6, seed=0):
    """Host CSR + sinogram + sensitivity + reference initial image for a preset.

    "cyl3d_tiny_dense" is a small cylinder (2 x 24 detectors, 40x40x8 voxels
    of 0.8 mm, 3x2 sub-rays) dense enough (> 96 nnz per row) to select the
    one-warp-per-row kernels for the forward projection."""
    if name == "cyl3d_rows32":
        # 2 x 32 detectors (2,016 rows) and 24x24x8 voxels (4,608 cols): both
        # multiples of 32, the shapes the reference's csr-vector grid assumes
        geo = pkg.geometry(32, 2, 20.0, 3.0, nx=24, ny=24, nz=8, vx=1.0, vy=1.0, vz=1.0, sub_t=2, sub_z=2,
                           width_t=1.0, width_z=0.8)
    elif name == "cyl3d_tiny_dense":
        geo = pkg.geometry(24, 2, 20.0, 3.0, nx=40, ny=40, nz=8, vx=0.8, vy=0.8, vz=0.8, sub_t=3, sub_z=2,
                           width_t=1.5, width_z=1.2)
    else:
        geo = pkg.preset(name)
    rp, c, v, cols = pkg.siddon_host(geo)
    from mlem_gb300 import synth
    xt = synth.phantom(geo, n_shapes, seed=seed + 1)
    g = synth.poisson_sinogram(synth.project_host(rp, c, v, xt), total, seed=seed + 2)
    norm = O.colsum(rp, c, v, cols, f64=True)
    f0 = np.full(cols, O.initial_value(g, norm), np.float32)
    return dict(rp=rp, col=c, val=v, cols=cols, g=g, norm=norm, f0=f0, xt=xt, geo=geo)
