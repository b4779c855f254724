"""Failure detection on the GPU without a fault: the short range's bounded
staging wait is made to run out (a barrier armed for copies that are never
issued, a 2 ms limit), the timeout word is set, and the host reads
CUCO_ERR_TIMEOUT; the context stays usable and the word is cleared."""
import numpy as np
import pytest

from cuco_gb300 import Box, BoxConfig, ics

pytestmark = pytest.mark.gpu

CUCO_ERR_TIMEOUT = 4


def test_staging_wait_times_out_and_the_box_keeps_working():
    ic = ics.zeldovich(16, 50.0, 49.0, 4)
    box = Box(BoxConfig(n=ic.n, pm_grid=32, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                        softening=2.8 * 0.03 * ic.boxsize / 16))
    box.set_state(ic.pos, ic.canonical_velocity())
    st = box.lib.cuco_box_selftest_timeout(box.h, 0.002)
    assert st == CUCO_ERR_TIMEOUT
    assert b"gave up" in box.lib.cuco_last_error()
    # the word was read and cleared; the next pass runs and reports nothing
    box.forces()
    box.sync()
    _, _, app, apm = box.get_state()
    assert np.isfinite(app).all() and np.isfinite(apm).all() and np.abs(app).sum() > 0
    assert box.lib.cuco_box_selftest_timeout(box.h, 2.0) == 1  # limits above 1 s are refused
    box.close()
