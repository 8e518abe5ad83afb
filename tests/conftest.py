import importlib
import json
import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parent.parent
GOLDEN = Path(__file__).resolve().parent / "golden"
PKG_NAME = "multirobot-pathplanning-benchmark_gb300"

if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))
if str(ROOT / "oracle") not in sys.path:
    sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300) and the built CUDA library")


def pkg(sub: str | None = None):
    name = PKG_NAME if sub is None else f"{PKG_NAME}.{sub}"
    return importlib.import_module(name)


def golden(name: str):
    if name.endswith(".json"):
        return json.loads((GOLDEN / name).read_text())
    return np.load(GOLDEN / name, allow_pickle=False)


@pytest.fixture(scope="session")
def oracle():
    import oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def cuda_lib():
    """The built CUDA library (compiled here if missing)."""
    build = pkg("build")
    build.build()
    return pkg("_lib").load()


@pytest.fixture(scope="session")
def gpu():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    build = pkg("build")
    build.build()
    pkg("_lib").load()
    return torch.device("cuda")
