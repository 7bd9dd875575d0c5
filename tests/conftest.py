import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs on the GB300)")


@pytest.fixture(scope="session")
def gpu_ctx():
    import metriko_gb300 as M
    ctx = M.Context(0)
    yield ctx
    ctx.close()


_ORACLE_CACHE = {}


def oracle_run(name, **kw):
    """Cached full oracle pipeline for a named workload."""
    from metriko_gb300 import meshgen
    from oracle import metriko_oracle as O
    key = (name, tuple(sorted(kw.items())))
    if key not in _ORACLE_CACHE:
        V, F, ratio, rs = meshgen.workload(name)
        _ORACLE_CACHE[key] = (V, F, ratio, rs, O.pipeline(V, F, ratio=ratio, round_seams=rs, **kw))
    return _ORACLE_CACHE[key]
