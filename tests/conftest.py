import os
import sys

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (sm_103a) and the built library")
    config.addinivalue_line("markers", "late: full-size and host-environment checks, run after the bit-exact "
                                       "parity tests of the session")


def pytest_collection_modifyitems(session, config, items):
    # the fast bit-exact parity tests first, the full-size workloads and the checks that
    # depend on the host (a second GPU process, a bundled LAPACK) after them, and the
    # test_zz_* files last of all (a run that stops at their first failure has run the rest)
    def rank(it):
        if os.path.basename(str(it.fspath)).startswith("test_zz_"):
            return 2
        return 1 if it.get_closest_marker("late") else 0

    items.sort(key=rank)
