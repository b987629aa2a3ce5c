"""The device's failure detectors fire, and no GPU is faulted or hung to make them.

Two detectors exist: the sticky status word's non-finite bit (a nodal velocity or
displacement that stopped being finite, set by the nodal update) and the contact pass's
bounded grid barrier (a wait that runs out sets the timeout bit and releases every block, and
the kernel returns). Here the first is driven by a NaN written from the host; the second by
lowering the barrier's wait limit to a couple of polls, so that a block that must wait at all
gives up at once. Neither needs a faulting access, a trap or a wait without end.
"""
import numpy as np
import pytest

from neofiz_gb300 import ExplicitSolver, _abi, scenes
from neofiz_gb300.solver import DeviceError, DeviceTimeout

pytestmark = pytest.mark.gpu


def test_nonfinite_velocity_sets_the_status_word(gpu_lib):
    g, _, _ = scenes.taylor_rod(ExplicitSolver, nr=4, nz=24)
    g.run(20)
    g.check()
    assert g.statusWord() == 0
    vr = g.velocityR()
    vr[7] = np.nan
    g.writeField(_abi.FIELD_VR, vr)
    g.run(3)
    g.synchronize()                 # the reference lets NaNs propagate: stepping goes on
    assert g.statusWord() & _abi.STATUS_NONFINITE
    with pytest.raises(DeviceError, match="not finite"):
        g.check()
    # the bit is sticky
    g.run(1)
    assert g.statusWord() & _abi.STATUS_NONFINITE


def test_contact_barrier_that_runs_out_is_reported(gpu_lib):
    g, _, _ = scenes.two_blocks(ExplicitSolver, speed=400.0)
    g.run(5)
    g.check()
    g.setWaitLimit(1, 1)
    seen = False
    for _ in range(5):
        g.run(1)
        try:
            g.synchronize()
        except DeviceTimeout:
            seen = True
            break
    assert seen, "a one-poll barrier wait never ran out"
    assert g.statusWord() & _abi.STATUS_TIMEOUT
    # every later run call and check reports it; the handle no longer steps
    with pytest.raises(DeviceTimeout):
        g.run(1)
    with pytest.raises(DeviceTimeout):
        g.runUntil(1.0)
    with pytest.raises(DeviceTimeout):
        g.check()
    steps = g.steps()
    with pytest.raises(DeviceTimeout):
        g.run(10)
    assert g.steps() == steps
    # the context is intact: a fresh handle steps normally and reproduces an undisturbed run
    a, _, _ = scenes.two_blocks(ExplicitSolver, speed=400.0)
    b, _, _ = scenes.two_blocks(ExplicitSolver, speed=400.0)
    a.run(200)
    b.setWaitLimit(0, 0)
    b.run(200)
    a.check()
    b.check()
    assert a.statusWord() == 0 and b.statusWord() == 0
    for f in (_abi.FIELD_UR, _abi.FIELD_UZ, _abi.FIELD_VR, _abi.FIELD_VZ):
        assert np.array_equal(a.readField(f).view(np.uint64), b.readField(f).view(np.uint64))


def test_wait_limits_are_validated(gpu_lib):
    g, _, _ = scenes.two_blocks(ExplicitSolver)
    with pytest.raises(ValueError, match=">= 0"):
        g.setWaitLimit(-1, 0)
