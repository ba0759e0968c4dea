"""The round-end smoke entry point: one small coupled scene on cuda:0, five
steps through the C ABI, checked against the FP64 oracle."""
import os
import sys

import pytest

pytestmark = pytest.mark.gpu


def test_smoke_runs():
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    if root not in sys.path:
        sys.path.insert(0, root)
    import __graft_entry__ as g
    g.smoke()
