"""Access to the golden fixtures and the seeded problems they were generated from."""
import os

import numpy as np

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")


def load_golden(name):
    return dict(np.load(os.path.join(HERE, name + ".npz")))


def golden_module():
    """tests/golden/make_golden.py as a module (its case lists)."""
    import importlib.util
    spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
    mod = importlib.util.module_from_spec(spec)
    spec.loader.exec_module(mod)
    return mod


def golden_problem(name):
    return golden_module().cases()[name]
