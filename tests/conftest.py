import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built library")


@pytest.fixture(scope="session")
def coeff_dir(tmp_path_factory):
    from crtmv3_gb300 import synthetic as sy
    d = str(tmp_path_factory.mktemp("coeffs"))
    for s in sy.SENSORS:
        sy.write_sensor_files(d, s)
    return d


@pytest.fixture(scope="session")
def gpu_lib():
    import torch
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from crtmv3_gb300 import build
    build.build()
    from crtmv3_gb300 import api
    api.library()
    return api
