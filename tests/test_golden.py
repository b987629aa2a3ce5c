"""The committed golden fixtures (tests/golden/, written from the oracle by make_golden.py):
the oracle must keep reproducing them, so a change to the oracle itself cannot pass unseen,
and the device must reproduce them bit for bit, independently of a live oracle run."""
import importlib.util
import json
import os

import numpy as np
import pytest

HERE = os.path.join(os.path.dirname(os.path.abspath(__file__)), "golden")
_spec = importlib.util.spec_from_file_location("make_golden", os.path.join(HERE, "make_golden.py"))
mg = importlib.util.module_from_spec(_spec)
_spec.loader.exec_module(mg)
with open(os.path.join(HERE, "golden.json")) as f:
    GOLDEN = json.load(f)


def check(solver_cls, name):
    build, steps = mg.SCENES[name]
    rec = GOLDEN["scenes"][name]
    assert rec["steps"] == steps
    s, mesh, _ = build(solver_cls)
    got = mg.trace(s, steps)
    for want, have in zip(rec["trace"], got):
        assert want["time"] == have["time"], f"{name} step {want['step']}: time"
        bad = [k for k in mg.FIELDS if want[k] != have[k]]
        assert not bad, f"{name} step {want['step']}: fields {bad} differ from the fixture"
    if name in mg.FULL:
        data = np.load(os.path.join(HERE, f"{name}_step{steps}.npz"))
        for field in mg.FULL[name]:
            a, b = s.readField(mg.FIELDS[field]), data[field]
            assert a.dtype == b.dtype and np.array_equal(a.view(np.uint8), b.view(np.uint8)), field
    return s


@pytest.mark.parametrize("name", list(mg.SCENES))
def test_oracle_reproduces_the_fixtures(name):
    from oracle.oracle import OracleSolver
    s = check(OracleSolver, name)
    if name == "perforation_1mm":
        assert s.erodedElements() > 0


@pytest.mark.gpu
@pytest.mark.parametrize("name", list(mg.SCENES))
def test_device_reproduces_the_fixtures(gpu_lib, name):
    from neofiz_gb300 import ExplicitSolver
    s = check(ExplicitSolver, name)
    assert s.statusWord() == 0
