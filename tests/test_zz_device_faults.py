"""Collected last: no bounded device-side wait (the raster's TMA tile loads)
gave up during the GPU tests that ran before."""
import pytest

pytestmark = pytest.mark.gpu


def test_no_device_wait_gave_up(cuda):
    import depix
    cuda.cuda.synchronize()
    assert depix.take_device_faults() == 0
    assert depix.take_device_faults() == 0  # cleared
