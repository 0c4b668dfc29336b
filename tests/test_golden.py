"""Golden fixtures (tests/golden/*.npz, made by tests/golden/make_golden.py from the oracle): the
oracle must keep reproducing them, and the GPU library must reproduce them bit for bit — canonical
DAG (node kinds, types/mask bits, leaf and LOD values, refcounts, child links, roots), live node
count, changed flags and get() answers."""
import os

import numpy as np
import pytest

HERE = os.path.dirname(os.path.abspath(__file__))
GOLDEN = os.path.join(HERE, "golden")

import importlib.util  # noqa: E402

_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(GOLDEN, "make_golden.py"))
make_golden = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(make_golden)


@pytest.mark.parametrize("name", make_golden.CASES)
def test_golden_fixture(lib, name):
    want = np.load(os.path.join(GOLDEN, name + ".npz"))
    got = make_golden.run_case(name, lib)
    assert set(want.files) == set(got)
    for k in want.files:
        np.testing.assert_array_equal(got[k], want[k], err_msg="%s: %s" % (name, k))
