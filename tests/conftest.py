import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def port():
    from oracle import oracle as O
    O.build_port()
    return O.port()


@pytest.fixture(scope="session")
def ref_oracle():
    from oracle import oracle as O
    r = O.reference("fp64")
    if r is None:
        pytest.skip("reference-compiled oracle not available on this machine")
    return r


def load_golden(name: str) -> dict:
    with np.load(GOLDEN / name, allow_pickle=False) as z:
        return {k: z[k] for k in z.files}


def workload_from_golden(g: dict):
    from sphexa_gb300.workloads import Workload
    fields = {k[3:]: g[k] for k in g if k.startswith("in_")}
    params = {k[6:]: g[k].item() for k in g if k.startswith("param_")}
    return Workload("golden", len(fields["x"]), g["box_in"], g["bc"], fields, params)


@pytest.fixture(scope="session")
def gpu_ctx():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from sphexa_gb300 import sph
    ctx = sph.Context(0)
    yield ctx
    ctx.close()
