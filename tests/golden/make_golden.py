"""Writes the golden fixtures of this directory from the oracle (the CPU restatement of the
reference's Java path). Run from the repository root:

    python tests/golden/make_golden.py

Three scenes, each checked by tests/test_golden.py on the oracle (CPU) and on the device:

* rod_10x60: the 10 x 60 axisymmetric Johnson-Cook rod on the Coulomb anvil (the plain FP64
  Taylor case): every nodal and point field after 1000 steps (rod_10x60_step1000.npz), and a
  SHA-256 of every field's bytes every 100 steps;
* perforation_1mm: the plane-strain perforation at 1 mm cells (contact, friction, damage,
  erosion, gravity, floor): the digests every 100 steps to 600, and the eroded set, contact
  masters and stick/slip states at 600 in full;
* tube_4x20: the pressurised tube (pressure edges, relaxation damping, full integration,
  damage): the digests every 100 steps to 600.

The digests are over little-endian IEEE doubles and int32/uint8 arrays, the same on x86-64
and aarch64 hosts.
"""
import hashlib
import json
import os
import sys

import numpy as np

HERE = os.path.dirname(os.path.abspath(__file__))
ROOT = os.path.dirname(os.path.dirname(HERE))
if ROOT not in sys.path:
    sys.path.insert(0, ROOT)

from neofiz_gb300 import _abi, scenes  # noqa: E402

FIELDS = {
    "ur": _abi.FIELD_UR, "uz": _abi.FIELD_UZ, "vr": _abi.FIELD_VR, "vz": _abi.FIELD_VZ,
    "fr": _abi.FIELD_FR, "fz": _abi.FIELD_FZ, "stress": _abi.FIELD_STRESS,
    "back": _abi.FIELD_BACK_STRESS, "eps": _abi.FIELD_PLASTIC_STRAIN,
    "work": _abi.FIELD_PLASTIC_WORK, "hgr": _abi.FIELD_HOURGLASS_R,
    "hgz": _abi.FIELD_HOURGLASS_Z, "dstrength": _abi.FIELD_DAMAGE_STRENGTH,
    "eroded": _abi.FIELD_ERODED, "wall_state": _abi.FIELD_WALL_STATE,
    "contact_master": _abi.FIELD_CONTACT_MASTER, "contact_state": _abi.FIELD_CONTACT_STATE,
}
SCENES = {
    "rod_10x60": (lambda cls: scenes.taylor_rod(cls), 1000),
    "perforation_1mm": (lambda cls: scenes.perforation(cls, cell=1.0e-3), 600),
    "tube_4x20": (lambda cls: scenes.tube(cls), 600),
}
EVERY = 100
FULL = {"rod_10x60": ["ur", "uz", "vr", "vz", "stress", "back", "eps", "work"],
        "perforation_1mm": ["eroded", "contact_master", "contact_state"]}


def digest(a: np.ndarray) -> str:
    return hashlib.sha256(np.ascontiguousarray(a).tobytes()).hexdigest()[:32]


def trace(solver, steps):
    """The scene's digests every EVERY steps, and the solver at the end."""
    out = []
    for k in range(EVERY, steps + 1, EVERY):
        solver.run(EVERY)
        row = {"step": k, "time": solver.time().hex()}
        for name, f in FIELDS.items():
            row[name] = digest(solver.readField(f))
        out.append(row)
    return out


def main():
    from oracle.oracle import OracleSolver
    record = {"generator": "oracle (oracle/refcpu.c), tests/golden/make_golden.py",
              "every": EVERY, "scenes": {}}
    for name, (build, steps) in SCENES.items():
        s, _, _ = build(OracleSolver)
        record["scenes"][name] = {"steps": steps, "trace": trace(s, steps)}
        if name in FULL:
            np.savez_compressed(os.path.join(HERE, f"{name}_step{steps}.npz"),
                                **{f: s.readField(FIELDS[f]) for f in FULL[name]})
        print(name, "done")
    with open(os.path.join(HERE, "golden.json"), "w") as f:
        json.dump(record, f, indent=1)


if __name__ == "__main__":
    main()
