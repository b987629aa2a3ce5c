"""BurstCase.run's measurement as a batch (nf_batch_set_burst), on the oracle: against a
restatement of BurstCase.loadCapacity/hoopStrain driven through the single-scene oracle."""
import math

import numpy as np
import pytest

from neofiz_gb300 import _abi, scenes
from oracle.oracle import OracleBatch, OracleSolver, math_fn


def _capacity_and_strain(s, mesh, mean_radius):
    """BurstCase.loadCapacity (BurstCase.java:533-553) and hoopStrain (:560-569), in the
    reference's order."""
    ur, uz = s.readField(_abi.FIELD_UR), s.readField(_abi.FIELD_UZ)
    sig = s.readField(_abi.FIELD_STRESS)
    r = [float(mesh.r[i] + ur[i]) for i in range(mesh.nodeCount)]
    z = [float(mesh.z[i] + uz[i]) for i in range(mesh.nodeCount)]
    conn = mesh.conn
    hoop = 0.0
    for e in range(mesh.elementCount):
        total = 0.0
        for k in range(4):
            i, j = int(conn[4 * e + k]), int(conn[4 * e + (k + 1) % 4])
            total += r[i] * z[j] - r[j] * z[i]
        hoop += float(sig[4 * e + 2]) / 1.0 * (0.5 * total)
    bore, low, high = min(r), min(z), max(z)
    capacity = hoop / (bore * (high - low))
    strain = math_fn("log", 0.5 * (min(r) + max(r)) / mean_radius)
    return capacity, strain


def _single(inst):
    s = OracleSolver(inst.mesh, inst.material, scenes.Formulation.AXISYMMETRIC,
                     scenes.Integration.REDUCED, scenes.Kinematics.FINITE_STRAIN, 1.0,
                     scenes.BURST_CFL)
    for n in inst.fixed_axial:
        s.fixAxial(int(n))
    s.setPressureRamp(*inst.pressure)
    s.setRelaxationDamping(*inst.damping)
    return s


def test_burst_samples_match_the_restated_measurement():
    inst = scenes.burst_instance()
    b = OracleBatch([inst], scenes.Formulation.AXISYMMETRIC, cfl=scenes.BURST_CFL)
    b.setBurst(scenes.BURST_SAMPLE_STEPS, 25.0e-3, scenes.BURST_PEAK_MARGIN, traceCapacity=40)
    b.run(max_steps=30 * scenes.BURST_SAMPLE_STEPS + 7)      # stops mid-sample: no sample
    trace = b.burstTrace()[0]
    res = b.burstResults()
    assert res["samples"][0] == 30 and not res["traversed"][0]
    s = _single(inst)
    peak = 0.0
    for n in range(30):
        s.run(scenes.BURST_SAMPLE_STEPS)
        cap, strain = _capacity_and_strain(s, inst.mesh, 25.0e-3)
        t, st, c, applied = trace[n]
        assert t == s.time() and c == cap and st == strain
        assert applied == s.borePressure()
        peak = max(peak, cap)
    assert res["peak_capacity"][0] == peak
    assert b.state()["steps"][0] == 30 * scenes.BURST_SAMPLE_STEPS + 7


def test_burst_pressure_closed_form_is_thin_wall_barlow_like():
    law = scenes.burst_material().johnsonCook
    p = scenes.burst_pressure(law, 2.0e-3, 25.0e-3)
    assert 1.7e7 < p < 1.9e7                                 # ~18.1 MPa for this tube
    # thinner wall, proportionally lower pressure
    assert abs(scenes.burst_pressure(law, 1.0e-3, 25.0e-3) / p - 0.5) < 1e-12


def test_burst_settings_are_checked():
    b = OracleBatch([scenes.burst_instance()], scenes.Formulation.AXISYMMETRIC,
                    cfl=scenes.BURST_CFL)
    with pytest.raises(ValueError):
        b.setBurst(250, 25e-3, margin=1.5)
    with pytest.raises(RuntimeError):
        b.burstResults()
