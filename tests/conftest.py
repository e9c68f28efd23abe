import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parents[1]
sys.path.insert(0, str(ROOT))
sys.path.insert(0, str(ROOT / "oracle"))


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libpqgb300.so")


@pytest.fixture(scope="session")
def pq():
    import __graft_entry__ as g

    return g.load_package()


@pytest.fixture(scope="session")
def O():
    import tn_oracle

    return tn_oracle


class _HostBackend:
    """numpy (FP64) backend used to exercise the product's host logic on CPU."""

    def __init__(self):
        import tn_oracle

        self._b = tn_oracle.OracleBackend()
        self.metrics = self._b.metrics

    def __getattr__(self, name):
        return getattr(self._b, name)

    def shape(self, label):
        return self._b.tensors[label].shape

    def view_tensor(self, view, node, bond_idx, bond_range):
        lo, hi = (bond_range.start, bond_range.stop - 1) if isinstance(bond_range, range) else bond_range
        return self._b.view_tensor(view, node, bond_idx, lo, hi)

    @property
    def tensors(self):
        return self._b.tensors


@pytest.fixture
def host_backend():
    return _HostBackend()
