"""The device film against the oracle's state: the same frames, value for value."""
import json

import numpy as np
import pytest

from neofiz_gb300 import ExplicitSolver, _abi, scenes
from neofiz_gb300 import film as F
from oracle.oracle import OracleSolver

pytestmark = pytest.mark.gpu


def _expected(o, mesh):
    """Film.capture's values from the oracle's state, in the reference accessors' order."""
    ur, uz = o.readField(_abi.FIELD_UR), o.readField(_abi.FIELD_UZ)
    eps = o.readField(_abi.FIELD_PLASTIC_STRAIN)
    sig = o.readField(_abi.FIELD_STRESS).reshape(-1, 4)
    sf = o.readField(_abi.FIELD_DAMAGE_STRENGTH)
    soft = o.readField(_abi.FIELD_DAMAGE_SOFTENING)
    vr, vz = o.readField(_abi.FIELD_VR), o.readField(_abi.FIELD_VZ)
    eroded = o.readField(_abi.FIELD_ERODED)
    fail = np.full(mesh.elementCount, 0.8)
    dmg = np.zeros_like(eps)
    on = sf > 0.0
    d = -soft[on] * (eps[on] - fail[on]) / sf[on]
    dmg[on] = np.where(d <= 0.0, 0.0, np.where(d >= 1.0, 1.0, d))
    s = sig / 1.0
    a, b, c = s[:, 0] - s[:, 1], s[:, 1] - s[:, 2], s[:, 2] - s[:, 0]
    mises = np.sqrt(0.5 * (a * a + b * b + c * c) + 3.0 * s[:, 3] * s[:, 3]) / 1e6
    conn = mesh.conn.reshape(-1, 4)
    spd = np.sqrt(vr * vr + vz * vz)
    speed = 0.25 * (((spd[conn[:, 0]] + spd[conn[:, 1]]) + spd[conn[:, 2]]) + spd[conn[:, 3]])
    return (mesh.r + ur, mesh.z + uz,
            [eps / 1.0, dmg / 1.0, mises, s[:, 2] / 1e6, speed], eroded == 0)


def test_device_film_matches_the_oracle_state():
    g, mesh, _ = scenes.two_blocks(ExplicitSolver, speed=400.0)
    o, _, _ = scenes.two_blocks(OracleSolver, speed=400.0)
    kinds = [F.PLASTIC_STRAIN, F.DAMAGE, F.VON_MISES_MPA, F.HOOP_STRESS_MPA, F.SPEED]
    film = F.Film(mesh, capacity=2).planar()       # capacity 2: frames spill to the host
    for k in kinds:
        film.colourBy(str(k), "", F.AUTO, F.AUTO, k)
    film.aliveIf(F.NOT_ERODED).readout("ke", lambda fr: fr.audit.kinetic_energy)
    expected, audits = [], []
    for _ in range(5):
        g.run(60)
        o.run(60)
        film.capture(g)
        expected.append(_expected(o, mesh) + (o.time(), o.steps(), o.erodedElements()))
        audits.append(o._auditC())
    frames = film.frames()
    assert len(frames) == 5
    for fr, (r, z, vals, live, t, n, er), au in zip(frames, expected, audits):
        assert np.array_equal(fr.r, r) and np.array_equal(fr.z, z)
        for k in range(len(kinds)):
            assert np.array_equal(fr.values[k], vals[k]), kinds[k]
        assert np.array_equal(fr.live.astype(bool), live)
        assert fr.time == t and fr.steps == n and fr.eroded == er
        # per-block partial sums against the oracle's serial sums
        np.testing.assert_allclose(fr.audit.kinetic_energy, au.kinetic_energy, rtol=1e-12)
        np.testing.assert_allclose(fr.audit.plastic_dissipation, au.plastic_dissipation,
                                   rtol=1e-12)
    assert max(float(np.max(fr.values[0])) for fr in frames) > 0.0
    doc = json.loads(film.json("two blocks"))
    assert len(doc["frames"]) == 5 and doc["frames"][4]["t"] == float(F.number(expected[4][4]))
    film.close()


def test_a_full_film_refuses_more_frames_through_the_c_abi(gpu_lib):
    import ctypes as C
    g, mesh, _ = scenes.two_blocks(ExplicitSolver)
    api = g._api
    kinds = np.array([F.PLASTIC_STRAIN], dtype=np.int32)
    out = C.c_void_p()
    assert api.film_create(g._handle, kinds.ctypes.data_as(_abi.c_int32_p), 1, 1,
                           C.byref(out)) == 0
    assert api.film_capture(out) == 0
    assert api.film_capture(out) == _abi.NF_ESTATE
    bad = np.array([99], dtype=np.int32)
    out2 = C.c_void_p()
    assert api.film_create(g._handle, bad.ctypes.data_as(_abi.c_int32_p), 1, 4,
                           C.byref(out2)) == _abi.NF_EINVAL
    api.film_destroy(out)
