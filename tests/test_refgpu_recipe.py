"""The recipe that compiles the reference's own kernels into cubins
(oracle/build_ref.py) and the launch table of tests/refgpu.py, checked on
the CPU: every source it names exists in the reference tree, every kernel
refgpu.py launches is a __global__ function of the file whose cubin it
loads (skipped where the reference tree is absent)."""
import importlib.util
import os
import re

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def _recipe():
    spec = importlib.util.spec_from_file_location("build_ref", os.path.join(ROOT, "oracle", "build_ref.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def _launches():
    """(cubin, kernel) pairs launched by tests/refgpu.py."""
    src = open(os.path.join(ROOT, "tests", "refgpu.py")).read()
    pairs = set()
    for fn in re.split(r"\ndef ", src)[1:]:
        mods = re.findall(r'module\("(\w+)"\)', fn)
        kers = re.findall(r'launch\(\s*"(\w+)"', fn)
        for m in mods:
            for k in kers:
                pairs.add((m, k))
    return pairs


def test_launch_table_names_known_cubins():
    rec = _recipe()
    pairs = _launches()
    assert len(pairs) >= 11
    assert {m for m, _ in pairs} <= set(rec.CUBINS)


def test_kernels_exist_in_reference_sources():
    rec = _recipe()
    if not os.path.isdir(os.path.join(rec.REF, "rendering", "src")):
        pytest.skip("reference tree absent")
    for m, k in _launches():
        text = open(os.path.join(rec.REF, rec.CUBINS[m])).read()
        assert re.search(r"__global__\s+void\s+" + k + r"\s*\(", text), (m, k)
    missing = [n for n in rec.CUBINS if not os.path.exists(rec.cubin_path(n))]
    if missing:
        pytest.skip(f"cubins not built yet: {missing}")
