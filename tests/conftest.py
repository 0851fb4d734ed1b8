import sys
from pathlib import Path

import numpy as np
import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a) and the built libffcz.so")


@pytest.fixture(scope="session")
def golden_huffman():
    d = np.load(GOLDEN / "huffman_reference.npz")
    names = sorted({k.split("__")[0] for k in d.files})
    return {n: {k.split("__")[1]: d[k] for k in d.files if k.startswith(n + "__")} for n in names}


@pytest.fixture(scope="session")
def cuda():
    import torch

    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    torch.cuda.set_device(0)
    import ffcz_gb300

    ffcz_gb300.lib()  # fails loudly when the extension is missing
    return torch
