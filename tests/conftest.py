import os
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)
sys.path.insert(0, os.path.join(ROOT, "tests"))

import __graft_entry__ as graft  # noqa: E402


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300, sm_103a)")


_built = False


def _ensure_built():
    global _built
    if not _built:
        graft.build()
        _built = True


@pytest.fixture(scope="session")
def pkg():
    _ensure_built()
    return graft.load_package()


@pytest.fixture(scope="session")
def oracle():
    _ensure_built()
    import oracle_bindings

    return oracle_bindings


def fixed_iter_params(pkg, n_iter, nu0):
    """All tolerances disabled: a fixed number of LM iterations."""
    return pkg.OptParams(num_iterations=n_iter, initial_lm_damping=nu0, function_tolerance=0.0,
                         gradient_tolerance=0.0, parameter_tolerance=0.0, max_consecutive_rejects=1 << 40,
                         solver=pkg.LinearSolverEnum.SchurBlockSparseLdlt)
