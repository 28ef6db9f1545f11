import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
sys.path.insert(0, ROOT)

import __graft_entry__ as ge  # noqa: E402

GOLDEN = os.path.join(ROOT, "tests", "golden")


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (runs through libor3.so)")
    config.addinivalue_line("markers", "reference: needs the reference's compiled sources (oracle/_ref)")


@pytest.fixture(scope="session")
def pkg():
    return ge.load_package()


@pytest.fixture(scope="session")
def oracle_mod():
    return ge.load_oracle()


@pytest.fixture(scope="session")
def orc(oracle_mod):
    return oracle_mod.CRestatement()


@pytest.fixture(scope="session")
def ref(oracle_mod):
    if not oracle_mod.reference_available():
        if os.path.isdir(os.path.join(oracle_mod.REFERENCE_SRC, "src")):
            oracle_mod.build_oracle(reference=True)
        else:
            pytest.skip("reference sources not present on this machine")
    return oracle_mod.Reference()


@pytest.fixture(scope="session")
def ctx(pkg):
    c = pkg.Context(0)
    yield c
    c.close()


def golden(name):
    return np.load(os.path.join(GOLDEN, name), allow_pickle=False)


def zscores(m1, se1, n1, m2, se2, n2, rel_floor=1e-3):
    """Per-pixel two-sample z of two Monte Carlo estimates of the same pixel.

    Under the null hypothesis both estimators have the same per-path
    distribution, so the per-path variance is pooled from both sides
    (a side that saw no light at a pixel has a zero sample variance, which
    would otherwise make its standard error vanish).  `rel_floor` adds the
    storage precision of the fixtures (float16 means, ~5e-4 relative) so
    noise-free pixels (e.g. the light seen in the mirror) compare by value.
    Pixels that are exactly zero on both sides are skipped.
    """
    m1 = m1.astype(np.float64)
    m2 = m2.astype(np.float64)
    v1 = se1.astype(np.float64) ** 2 * n1
    v2 = se2.astype(np.float64) ** 2 * n2
    vp = (n1 * v1 + n2 * v2) / (n1 + n2)
    se = np.sqrt(vp * (1.0 / n1 + 1.0 / n2) + (rel_floor * np.maximum(np.abs(m1), np.abs(m2))) ** 2)
    ok = se > 0
    return (m1[ok] - m2[ok]) / se[ok]


def moments_to_mean_se(s, q, n):
    m = s / n
    var = np.maximum(q / n - m * m, 0.0) / n
    return m, np.sqrt(var)
