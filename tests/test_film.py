"""The film writer (render/Film.java) on the CPU: number formatting, the auto ramp and the
file layout. The device capture itself is checked in test_film_gpu.py."""
import json
import math
import types

import numpy as np

from neofiz_gb300 import _abi
from neofiz_gb300 import film as F
from neofiz_gb300.mesh import QuadMesh


def test_numbers_follow_javas_six_significant_figures():
    # Film.number (Film.java:352-362) over String.format("%.6g"): shortest digits rounded
    # half up, fixed notation from 1e-4 up to 1e6, trailing zeros trimmed, bare exponent
    cases = {0.0: "0", float("nan"): "0", float("inf"): "0", 1.0: "1", 0.5: "0.5",
             -0.5: "-0.5", 100.0: "100", 123456.7: "123457", 1234567.5: "1.23457e6",
             999999.5: "1e6", 0.000123456789: "0.000123457", 0.00009999996: "0.0001",
             0.15: "0.15", 1.234565e-5: "1.23457e-5", 2.0 / 3.0: "0.666667",
             -7.5e-7: "-7.5e-7", 3.0e8: "3e8", 0.025: "0.025", 1e-9: "1e-9"}
    for v, text in cases.items():
        assert F.number(v) == text, (v, F.number(v), text)


def test_auto_ramp_clips_half_a_per_cent():
    col = [np.arange(1000, dtype=np.float64)]
    low, high, peak = F.observed_range(col)
    assert (low, high, peak) == (0.0, 994.0, 999.0)      # floor(1000 * 0.005) = 5 above
    assert F.observed_range([np.arange(10.0)]) == (0.0, 9.0, 9.0)   # nothing clipped
    assert F.observed_range([np.full(4, np.nan)]) == (0.0, 1.0, 1.0)
    lo, hi, pk = F.observed_range([np.full(3, 2.0)])
    assert lo == 2.0 and hi == 2.0 + max(1e-9, 2.0 * 1e-6) and pk == 2.0


def _frame(t, r, z, values, live, ke):
    info = types.SimpleNamespace(time=t, steps=7, eroded=0, contact_pairs=3, pressure=0.0)
    audit = _abi.Audit()
    audit.kinetic_energy = ke
    return F.Frame(info, audit, np.asarray(r), np.asarray(z), np.asarray(values),
                   np.asarray(live))


def test_file_layout_is_the_references():
    mesh = QuadMesh.solidCylinder(1.0, 2.0, 1, 2)
    f = (F.Film(mesh).planar()
         .colourBy("body", "", 0.0, 1.0, np.array([1.0, 0.0]))
         .colourBy("plastic strain", "", F.AUTO, F.AUTO, F.PLASTIC_STRAIN)
         .aliveIf(F.NOT_ERODED)
         .readout("time, us", lambda fr: 1e6 * fr.time)
         .readout("kinetic energy, J", lambda fr: fr.audit.kinetic_energy))
    r = mesh.r + 0.1
    f._frames = [_frame(1e-6, r, mesh.z, [[0.25, 0.5]], [1, 0], 2.5),
                 _frame(2e-6, r, mesh.z, [[0.3, 0.75]], [1, 1], 1.25)]
    text = f.json('a "quoted" title')
    assert text.startswith('{"title":"a \\"quoted\\" title","axisymmetric":false,"nodes":6,')
    doc = json.loads(text)
    assert list(doc) == ["title", "axisymmetric", "nodes", "elements", "conn", "boundary",
                         "fields", "readouts", "frames"]
    assert doc["conn"] == [int(c) for c in mesh.conn]
    assert doc["boundary"] == [int(c) for c in mesh.surface()[0]]
    assert doc["fields"][0] == {"name": "body", "units": "", "low": 0, "high": 1, "peak": 1,
                                "auto": False}
    assert doc["fields"][1]["auto"] is True and doc["fields"][1]["low"] == 0.25
    assert doc["readouts"] == ["time, us", "kinetic energy, J"]
    fr = doc["frames"][1]
    assert list(fr) == ["t", "r", "z", "v", "s", "live"]
    assert fr["t"] == 2e-6 and fr["s"] == [2, 1.25] and fr["live"] == "11"
    assert fr["v"] == [[1, 0], [0.3, 0.75]]
    assert fr["r"] == [float(F.number(x)) for x in r]
