import os
import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 (sm_103a) GPU")


def _build_once():
    import importlib.util
    spec = importlib.util.spec_from_file_location("hq_build", ROOT / "hyquas_gb300" / "build.py")
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    mod.build()
    import subprocess
    subprocess.run(["make", "-C", str(ROOT / "oracle"), "liboracle.so"], check=True,
                   capture_output=True)


_build_once()


def gpu_available() -> bool:
    try:
        import hyquas_gb300 as hq
        hq.init(0)
        return True
    except Exception:
        return False


@pytest.fixture(scope="session")
def hq():
    import hyquas_gb300
    hyquas_gb300.init(0)
    return hyquas_gb300


@pytest.fixture(scope="session")
def oracle():
    import oracle as O
    return O
