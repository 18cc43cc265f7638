import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for sub in ("poets-dpd_gb300", "oracle", "tests"):
    p = os.path.join(ROOT, sub)
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")
    config.addinivalue_line("markers", "slow: long-running statistical checks")


def pytest_addoption(parser):
    parser.addoption("--host-direct", default=None, choices=["0", "1"],
                     help="force the engines' host_direct config (0: the attach and read-backs "
                          "through pinned staging and DMA even where the device reaches host "
                          "memory), to run the GPU tests on either copy path")


@pytest.fixture(autouse=True)
def _host_direct(request, monkeypatch):
    value = request.config.getoption("--host-direct")
    if value is None:
        yield
        return
    import pdpd_engine as E

    eng_init, srv_init = E.GB300DPDEngine.__init__, E.GB300DPDServer.__init__

    def engine(self, *a, **k):
        eng_init(self, *a, **k)
        self.SetConfigEntry("host_direct", value)

    def server(self, *a, **k):
        srv_init(self, *a, **k)
        self.config("host_direct", value)

    monkeypatch.setattr(E.GB300DPDEngine, "__init__", engine)
    monkeypatch.setattr(E.GB300DPDServer, "__init__", server)
    yield
