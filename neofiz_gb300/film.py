"""Film: deformed geometry captured over a run (render/Film.java), with the capture on the GPU.

The reference's ``Film`` copies the solver's state for every frame and evaluates its field
lambdas element by element on the host. Here ``capture`` enqueues the frame on the device
(``nf_film_capture``: deformed positions, the device fields, live flags, scalars and audit
partial sums, in FP64 as the reference holds them) and nothing comes back until
``json``/``write`` reads every frame at once. Fields may also be per-element
arrays (constant over the run, e.g. which body an element belongs to) or callables of the
solver, which are evaluated on the host at capture time as the reference does.

The file layout is the reference's (Film.json, Film.java:230-300): the viewer reads it
unchanged.
"""
from __future__ import annotations

import ctypes as C
import math
from decimal import ROUND_HALF_UP, Decimal
from typing import Callable, List, Optional, Union

import numpy as np

from . import _abi
from .solver import DeviceError

AUTO = float("nan")

# device fields (NF_FILM_*)
PLASTIC_STRAIN = _abi.FILM_PLASTIC_STRAIN
DAMAGE = _abi.FILM_DAMAGE
VON_MISES_MPA = _abi.FILM_VON_MISES_MPA
HOOP_STRESS_MPA = _abi.FILM_HOOP_STRESS_MPA
SPEED = _abi.FILM_SPEED
NOT_ERODED = "not eroded"

RAMP_CLIP = 0.005


def number(value: float) -> str:
    """Film.number (Film.java:352-362): Java's %.6g -- the double's shortest decimal digits
    (as Double.toString gives them) rounded half up to six significant figures, fixed notation
    for 1e-4 <= |rounded| < 1e6 -- with trailing zeros trimmed and a bare exponent."""
    if not math.isfinite(value) or value == 0.0:
        return "0"
    d = Decimal(repr(float(value)))
    sign = "-" if d < 0 else ""
    d = abs(d)
    exp = d.adjusted()
    q = d.scaleb(-exp).quantize(Decimal("1.00000"), rounding=ROUND_HALF_UP)
    if q >= 10:
        exp += 1
        q = d.scaleb(-exp).quantize(Decimal("1.00000"), rounding=ROUND_HALF_UP)
    if -4 <= exp < 6:
        frac = 5 - exp
        text = f"{q.scaleb(exp):.{frac}f}"
        return sign + (_trim(text) if "." in text else text)
    return sign + _trim(f"{q:.5f}") + "e" + str(exp)


def _trim(text: str) -> str:
    end = len(text)
    while end > 0 and text[end - 1] == "0":
        end -= 1
    if end > 0 and text[end - 1] == ".":
        end -= 1
    return text[:end]


def _escape(text: str) -> str:
    return text.replace("\\", "\\\\").replace('"', '\\"')


def observed_range(columns: List[np.ndarray]):
    """Film.observedRange (Film.java:306-334): low, a top that clips half a per cent of the
    samples, and the peak."""
    finite = [c[np.isfinite(c)] for c in columns]
    n = int(sum(f.size for f in finite))
    if n == 0:
        return 0.0, 1.0, 1.0
    allv = np.sort(np.concatenate(finite).astype(np.float64))
    low, peak = float(allv[0]), float(allv[-1])
    above = int(math.floor(n * RAMP_CLIP))
    high = float(allv[max(0, n - 1 - above)])
    if high <= low:
        high = peak
    if high - low < 1e-12 * max(1.0, abs(high)):
        return low, low + max(1e-9, abs(low) * 1e-6), peak
    return low, high, peak


class Frame:
    """One captured frame as read back: time, steps, eroded, contact_pairs, pressure and the
    audit (an ``_abi.Audit``) are what readouts are computed from."""

    def __init__(self, info, audit, r, z, values, live):
        self.time = info.time
        self.steps = info.steps
        self.eroded = info.eroded
        self.contact_pairs = info.contact_pairs
        self.pressure = info.pressure
        self.audit = audit
        self.r, self.z, self.values, self.live = r, z, values, live


class Film:
    def __init__(self, mesh, capacity: int = 256):
        self.mesh = mesh
        self.capacity = int(capacity)
        self.axisymmetric = True
        self.fields = []              # (name, units, low, high, source)
        self.readouts = []            # (name, fn(frame))
        self.alive = None
        self._device = None           # (api, handle, solver)
        self._host = []               # per capture: host-evaluated field columns and live
        self._frames: List[Frame] = []

    # ------------------------------------------------------------------ building
    def planar(self) -> "Film":
        self.axisymmetric = False
        return self

    def colourBy(self, name: str, units: str, low: float, high: float,
                 value: Union[int, np.ndarray, Callable]) -> "Film":
        self.fields.append((name, units, float(low), float(high), value))
        return self

    def aliveIf(self, test) -> "Film":
        self.alive = test
        return self

    def readout(self, name: str, value: Callable[[Frame], float]) -> "Film":
        self.readouts.append((name, value))
        return self

    # ------------------------------------------------------------------ capture
    def _device_kinds(self):
        return [v for (_, _, _, _, v) in self.fields if isinstance(v, (int, np.integer))]

    def _check(self, st):
        if st:
            api, handle, _ = self._device
            msg = api.film_last_error(handle)
            raise DeviceError(msg.decode() if msg else f"status {st}")

    def capture(self, solver) -> None:
        if self._device is None:
            api = solver._api
            kinds = np.array(self._device_kinds(), dtype=np.int32)
            out = C.c_void_p()
            st = api.film_create(solver._handle, kinds.ctypes.data_as(_abi.c_int32_p),
                                 int(kinds.size), self.capacity, C.byref(out))
            if st:
                msg = api.film_last_error(None)
                raise DeviceError(msg.decode() if msg else f"status {st}")
            self._device = (api, out, solver)
        api, handle, owner = self._device
        if owner is not solver:
            raise ValueError("a film captures one solver")
        n = C.c_int32()
        self._check(api.film_frames(handle, C.byref(n)))
        if n.value >= self.capacity:
            self._spill()
        host = {}
        for k, (_, _, _, _, v) in enumerate(self.fields):
            if callable(v):
                host[k] = np.asarray(v(solver), dtype=np.float64)
        if callable(self.alive):
            host["live"] = np.asarray(self.alive(solver), dtype=bool)
        self._host.append(host)
        self._check(api.film_capture(handle))

    def _spill(self) -> None:
        """Reads the device frames into host memory and empties the device film."""
        if self._device is None:
            return
        api, handle, solver = self._device
        n = C.c_int32()
        self._check(api.film_frames(handle, C.byref(n)))
        count = n.value
        if count == 0:
            return
        N, E = self.mesh.nodeCount, self.mesh.elementCount
        F = len(self._device_kinds())
        r = np.empty((count, N), np.float64)
        z = np.empty((count, N), np.float64)
        vals = np.empty((count, max(F, 1), E), np.float64)
        live = np.empty((count, E), np.uint8)
        info = (_abi.FilmInfo * count)()
        audits = (_abi.Audit * count)()
        f64 = _abi.c_double_p
        self._check(api.film_read(handle, r.ctypes.data_as(f64), z.ctypes.data_as(f64),
                                  vals.ctypes.data_as(f64),
                                  live.ctypes.data_as(C.POINTER(C.c_uint8)), info, audits))
        for k in range(count):
            self._frames.append(Frame(info[k], audits[k], r[k], z[k], vals[k, :F], live[k]))
        self._check(api.film_clear(handle))

    def frames(self) -> List[Frame]:
        self._spill()
        return self._frames

    def size(self) -> int:
        n = len(self._frames)
        if self._device is not None:
            c = C.c_int32()
            self._check(self._device[0].film_frames(self._device[1], C.byref(c)))
            n += c.value
        return n

    def close(self) -> None:
        if self._device is not None:
            self._device[0].film_destroy(self._device[1])
            self._device = None

    def __del__(self):
        try:
            self.close()
        except Exception:
            pass

    # ------------------------------------------------------------------ output
    def _columns(self, frames: List[Frame]):
        """Per field, per frame, the element values in the order fields were added."""
        cols = []
        dev = 0
        for k, (_, _, _, _, v) in enumerate(self.fields):
            per = []
            for i, fr in enumerate(frames):
                if isinstance(v, (int, np.integer)):
                    per.append(fr.values[dev])
                elif callable(v):
                    per.append(self._host[i][k])
                else:
                    per.append(np.asarray(v, dtype=np.float64))
            if isinstance(v, (int, np.integer)):
                dev += 1
            cols.append(per)
        return cols

    def json(self, title: str) -> str:
        frames = self.frames()
        cols = self._columns(frames)
        out = [f'{{"title":"{_escape(title)}"',
               f',"axisymmetric":{"true" if self.axisymmetric else "false"}',
               f',"nodes":{self.mesh.nodeCount}', f',"elements":{self.mesh.elementCount}']
        out.append(',"conn":[' + ",".join(str(int(c)) for c in self.mesh.conn) + "]")
        boundary = self.mesh.surface()[0]
        out.append(',"boundary":[' + ",".join(str(int(c)) for c in boundary) + "]")
        fl = []
        for k, (name, units, low, high, _) in enumerate(self.fields):
            auto = math.isnan(low) or math.isnan(high)
            rng = observed_range(cols[k]) if auto else (low, high, high)
            fl.append(f'{{"name":"{_escape(name)}","units":"{_escape(units)}"'
                      f',"low":{number(rng[0])},"high":{number(rng[1])}'
                      f',"peak":{number(rng[2])},"auto":{"true" if auto else "false"}}}')
        out.append(',"fields":[' + ",".join(fl) + "]")
        out.append(',"readouts":[' + ",".join(f'"{_escape(n)}"' for n, _ in self.readouts)
                   + "]")
        fr_text = []
        for i, fr in enumerate(frames):
            parts = [f'{{"t":{number(fr.time)}']
            parts.append(',"r":[' + ",".join(number(float(x)) for x in fr.r) + "]")
            parts.append(',"z":[' + ",".join(number(float(x)) for x in fr.z) + "]")
            parts.append(',"v":[' + ",".join(
                "[" + ",".join(number(float(x)) for x in cols[k][i]) + "]"
                for k in range(len(self.fields))) + "]")
            parts.append(',"s":[' + ",".join(number(float(fn(fr))) for _, fn in self.readouts)
                         + "]")
            if self.alive is not None:
                live = (fr.live if self.alive == NOT_ERODED else self._host[i]["live"])
                parts.append(',"live":"' + "".join("1" if x else "0" for x in live) + '"')
            parts.append("}")
            fr_text.append("".join(parts))
        out.append(',"frames":[' + ",".join(fr_text) + "]}")
        return "".join(out)

    def write(self, path: str, title: str) -> str:
        """Film.write (Film.java:188-205): the two globals a viewer page reads."""
        with open(path, "w", encoding="utf-8") as f:
            f.write("window.NEOFIZ_FILM = ")
            f.write(self.json(title))
            f.write(";\n")
            f.write("(window.NEOFIZ_FILMS = window.NEOFIZ_FILMS || []).push(window.NEOFIZ_FILM);\n")
        return path
