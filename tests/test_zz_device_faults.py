"""Collected after the other GPU tests (only test_zz_no_alloc.py comes later
and checks its own calls): no bounded device-side wait for a TMA tile load
(raster, graph or heuristics stage) gave up during the tests that ran
before. test_gpu_failures.py makes one give up on purpose and clears the
flag it set."""
import pytest

pytestmark = pytest.mark.gpu


def test_no_device_wait_gave_up(cuda):
    import depix
    cuda.cuda.synchronize()
    assert depix.take_device_faults() == 0
    assert depix.take_device_faults() == 0  # cleared
