import json
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
GOLDEN = ROOT / "tests" / "golden"


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")


@pytest.fixture(scope="session")
def golden():
    return json.loads((GOLDEN / "golden.json").read_text())


@pytest.fixture(scope="session")
def port():
    from oracle.pyoracle import Port
    return Port()


@pytest.fixture(scope="session")
def blocks_input(golden):
    from nebc7_gb300 import synth
    n = golden["blocks"]["n"]
    seed = golden["blocks"]["seed"]
    cells, masks = synth.random_blocks(n, seed)
    starts = synth.random_start_blocks(n, seed + 1)
    return cells, masks, starts


@pytest.fixture(scope="session")
def native():
    """The CUDA library, built in-tree if needed; only for gpu tests."""
    import nebc7_gb300
    nebc7_gb300.build()
    return nebc7_gb300.load()
