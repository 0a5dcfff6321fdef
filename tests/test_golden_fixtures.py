"""The committed golden fixtures are what their generator makes from the
reference tree: regenerated into a scratch folder, byte for byte the same.
The tree's location comes from RETROFIRE_REF (else the generator's
default); skipped where it is absent."""
import filecmp
import importlib.util
import os

import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")


def _generator():
    spec = importlib.util.spec_from_file_location("make_goldens", os.path.join(GOLDEN, "make_goldens.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def test_fixtures_regenerate_identically():
    gen = _generator()
    ref = os.environ.get("RETROFIRE_REF") or gen.DEFAULT_REF
    if not os.path.isdir(ref):
        pytest.skip("reference tree not available")
    out = os.path.join(os.path.dirname(HERE), "retrofire_gb300", "_build", "goldens")
    os.makedirs(out, exist_ok=True)
    gen.main(ref, out)
    for name in ("textured_quad.npz", "triangle.npz", "reference_vectors.json"):
        assert filecmp.cmp(os.path.join(out, name), os.path.join(GOLDEN, name), shallow=False), name
