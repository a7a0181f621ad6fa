import json
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
sys.path.insert(0, ROOT)


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a CUDA GPU (GB300) and the built CUDA library")
    config.addinivalue_line("markers", "slow: long-running")


@pytest.fixture(scope="session")
def golden_lists():
    return np.load(os.path.join(GOLDEN, "lists.npz"))


@pytest.fixture(scope="session")
def golden_lists_meta():
    with open(os.path.join(GOLDEN, "lists_meta.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_sigma():
    return np.load(os.path.join(GOLDEN, "sigma.npz"))


@pytest.fixture(scope="session")
def golden_rdm():
    return np.load(os.path.join(GOLDEN, "rdm.npz"))


@pytest.fixture(scope="session")
def golden_rdm3():
    with open(os.path.join(GOLDEN, "rdm3_checksums.json")) as f:
        meta = json.load(f)
    return meta, np.load(os.path.join(GOLDEN, "rdm3.npz"))


def rdm_checksum_matches(a, ref, seed, tol=1e-12):
    """a against a checksum of tests/golden/make_golden.py:rdm_checksum (same seed recipe)."""
    a = np.asarray(a).reshape(-1)
    if ref["size"] == 0:
        return a.size == 0
    if a.size != ref["size"]:
        return False
    rng = np.random.default_rng(seed)
    w = rng.normal(size=a.size)
    idx = np.sort(rng.choice(a.size, size=min(64, a.size), replace=False))
    scale = max(1.0, ref["norm"])
    return (idx.tolist() == ref["idx"] and abs(float(np.linalg.norm(a)) - ref["norm"]) <= tol * scale
            and abs(float(a @ w) - ref["dot_w"]) <= tol * scale * np.sqrt(a.size)
            and np.abs(a[idx] - np.array(ref["vals"])).max() <= tol * scale)


@pytest.fixture(scope="session")
def golden_checksums():
    with open(os.path.join(GOLDEN, "sigma_checksums.json")) as f:
        return json.load(f)


@pytest.fixture(scope="session")
def golden_davidson():
    with open(os.path.join(GOLDEN, "davidson.json")) as f:
        return json.load(f)


def sigma_cases(golden):
    keys = sorted({"_".join(k.split("_")[:3]) for k in golden.files})
    return [tuple(int(x) for x in k.split("_")) for k in keys]


def list_cases(golden):
    keys = sorted({"_".join(k.split("_")[:3]) for k in golden.files})
    return [tuple(int(x) for x in k.split("_")) for k in keys]


@pytest.fixture(scope="session")
def cuda():
    torch = pytest.importorskip("torch")
    if not torch.cuda.is_available():
        pytest.skip("no CUDA device")
    from forte2_gb300.build import LIB_PATH

    if not os.path.exists(LIB_PATH):
        from forte2_gb300.build import build

        build()
    return torch
