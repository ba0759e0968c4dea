"""Failure detection without a GPU fault: the bounded grid barrier of the
cooperative sorts gives up when a block never arrives, records the timeout in
the device status and returns, and the context stays usable."""
import pytest

pytestmark = pytest.mark.gpu


def test_barrier_completes_when_every_block_arrives(ds):
    assert ds.selftest_barrier(0, missing=0) == 0


def test_barrier_wait_runs_out_and_reports(ds):
    st = ds.selftest_barrier(0, missing=1)
    assert st & 128, f"status {st}: the wait for a block that never arrives should run out"
    # the context is still usable afterwards
    assert ds.selftest_barrier(0, missing=0) == 0
