import sys
from pathlib import Path

import pytest

ROOT = Path(__file__).resolve().parent.parent
if str(ROOT) not in sys.path:
    sys.path.insert(0, str(ROOT))

import __graft_entry__  # noqa: E402

__graft_entry__.package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built libkhronos_gb300.so")


@pytest.fixture(scope="session")
def kh():
    import khronos_gb300

    return khronos_gb300


@pytest.fixture(scope="session")
def oracle():
    import oracle.oracle as orc

    orc.build()
    return orc


@pytest.fixture(scope="session")
def gpu_lib():
    """The CUDA library, built for this machine; fails loudly if it cannot load."""
    from khronos_gb300 import _abi, build

    build.build()
    return _abi.load()


def rel_l2(a, b):
    import numpy as np

    nb = np.linalg.norm(b)
    if nb == 0:
        return float(np.linalg.norm(a))
    return float(np.linalg.norm(a - b) / nb)


def field_errors(fa, fb):
    """Relative L2 error of each of the 6 components, normalised by the norm of
    the whole E or H vector field it belongs to (components that vanish by
    symmetry carry only rounding noise, so a per-component ratio is noise/noise).
    Values are rescaled first so fields that have grown large do not overflow."""
    import numpy as np

    out = []
    for grp in ((0, 1, 2), (3, 4, 5)):
        scale = max(max(float(np.max(np.abs(fb[c]))) for c in grp), 1e-300)
        ref = np.sqrt(sum(float(np.sum((fb[c] / scale) ** 2)) for c in grp))
        for c in grp:
            err = float(np.linalg.norm((fa[c] - fb[c]) / scale))
            out.append(err / ref if ref > 0 else err)
    return out


def dft_errors(da, db):
    """Relative L2 error of each DFT array, normalised by the largest monitor norm."""
    import numpy as np

    scale = max(max(float(np.linalg.norm(b)) for b in db), 1e-300)
    return [float(np.linalg.norm(a - b)) / scale for a, b in zip(da, db)]
