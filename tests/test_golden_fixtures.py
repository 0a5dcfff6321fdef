"""The committed golden fixtures are what their generator makes from the
reference tree: regenerated into a scratch folder, byte for byte the same.
Skipped where the reference tree is not mounted."""
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
    if not os.path.isdir(gen.DEFAULT_REF):
        pytest.skip("reference tree not mounted")
    out = os.path.join(os.path.dirname(HERE), "retrofire_gb300", "_build", "goldens")
    os.makedirs(out, exist_ok=True)
    gen.main(gen.DEFAULT_REF, out)
    for name in ("textured_quad.npz", "triangle.npz", "reference_vectors.json"):
        assert filecmp.cmp(os.path.join(out, name), os.path.join(GOLDEN, name), shallow=False), name
