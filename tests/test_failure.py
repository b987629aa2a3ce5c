"""Failure detection on the CPU: the oracle's twin of the device's non-finite check, and the
wait-limit setter's validation (the oracle never waits). The device side is in
test_failure_gpu.py."""
import numpy as np
import pytest

from neofiz_gb300 import _abi, scenes
from neofiz_gb300.solver import DeviceError
from oracle.oracle import OracleSolver


def test_oracle_check_flags_a_nonfinite_velocity():
    o, _, _ = scenes.taylor_rod(OracleSolver, nr=2, nz=8)
    o.run(5)
    o.check()
    vz = o.velocityZ()
    vz[3] = np.inf
    o.writeField(_abi.FIELD_VZ, vz)
    with pytest.raises(DeviceError, match="not finite"):
        o.check()


def test_oracle_wait_limit_validation():
    o, _, _ = scenes.taylor_rod(OracleSolver, nr=2, nz=8)
    o.setWaitLimit(0, 0)
    with pytest.raises(ValueError, match=">= 0"):
        o.setWaitLimit(0, -5)


def test_oracle_grid_slots_validation():
    o, _, _ = scenes.taylor_rod(OracleSolver, nr=2, nz=8)
    o.setGridSlots(0)
    o.setGridSlots(64)
    with pytest.raises(ValueError, match=r"\[0, 64\]"):
        o.setGridSlots(65)
