"""Shared test setup: registers the `gpu` marker, loads the package directory
`abea-opencl_gb300/` as the module `abea_gb300`, and loads the golden fixtures."""
import importlib.util
import os
import sys

import numpy as np
import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
GOLDEN = os.path.join(ROOT, "tests", "golden")
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)


def load_package():
    if "abea_gb300" in sys.modules:
        return sys.modules["abea_gb300"]
    pkg_dir = os.path.join(ROOT, "abea-opencl_gb300")
    spec = importlib.util.spec_from_file_location(
        "abea_gb300", os.path.join(pkg_dir, "__init__.py"), submodule_search_locations=[pkg_dir])
    m = importlib.util.module_from_spec(spec)
    sys.modules["abea_gb300"] = m
    spec.loader.exec_module(m)
    return m


abea = load_package()


def pytest_configure(config):
    config.addinivalue_line("markers", "gpu: needs a GB300 and the built libabea.so")


def batch_from_npz(d):
    """Rebuilds a flattened Batch from a fixture written by make_golden.py."""
    from abea_gb300.types import EVENT_DTYPE, MODEL_DTYPE, SCALINGS_DTYPE, Batch
    ev = np.zeros(len(d["event_mean"]), dtype=EVENT_DTYPE)
    ev["mean"] = d["event_mean"]
    return Batch(read=d["read"], read_ptr=d["read_ptr"], read_len=d["read_len"], events=ev,
                 event_ptr=d["event_ptr"], n_events=d["n_events"],
                 scalings=np.ascontiguousarray(d["scalings"]).view(SCALINGS_DTYPE).reshape(-1),
                 model=np.ascontiguousarray(d["model"]).view(MODEL_DTYPE).reshape(-1))


def split_fixture_pairs(flat, counts):
    from abea_gb300.types import PAIR_DTYPE
    flat = np.ascontiguousarray(flat).view(PAIR_DTYPE).reshape(-1)
    out, p = [], 0
    for c in counts:
        c = max(int(c), 0)
        out.append(flat[p:p + c])
        p += c
    return out


@pytest.fixture(scope="session")
def dump_subset():
    d = np.load(os.path.join(GOLDEN, "dump_small_subset.npz"))
    return batch_from_npz(d), split_fixture_pairs(d["golden_pairs"], d["golden_counts"])


@pytest.fixture(scope="session")
def ref_synthetic():
    d = np.load(os.path.join(GOLDEN, "ref_synthetic.npz"))
    b = batch_from_npz(d)
    names = [str(x) for x in d["names"]]
    bands = {n: (d[f"bands__{n}"], d[f"trace__{n}"], d[f"bll__{n}"]) for n in names if f"bands__{n}" in d}
    return b, names, d["ref_counts"], split_fixture_pairs(d["ref_pairs"], d["ref_counts"]), bands


@pytest.fixture(scope="session")
def oracle_mod():
    from oracle import oracle
    oracle.build()
    return oracle
