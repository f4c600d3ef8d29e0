import os
import runpy
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
for p in (os.path.join(ROOT, "mpas-o-flecsi-2.0_gb300"), os.path.join(ROOT, "oracle"),
          os.path.join(ROOT, "tests")):
    if p not in sys.path:
        sys.path.insert(0, p)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA device (GB300); parity tests of the CUDA path")


@pytest.fixture(scope="session", autouse=True)
def built():
    """Builds libmpaso and the oracle libraries (incremental: a no-op when current)."""
    runpy.run_path(os.path.join(ROOT, "mpas-o-flecsi-2.0_gb300", "build.py"), run_name="mpaso_build")["build"]()
    ob = runpy.run_path(os.path.join(ROOT, "oracle", "build.py"), run_name="oracle_build")
    ob["build_restatement"]()
    try:  # the shim-built reference: tests that need it skip when it is absent
        ob["build_ref"]()
    except Exception as e:  # noqa: BLE001
        print(f"warning: reference build failed: {e}", file=sys.stderr)
    return True
