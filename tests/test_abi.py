"""The C-ABI library: it builds, loads without a GPU, and exports every declared entry point."""
import ctypes
import os
import re
import subprocess
import sys

import pytest

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))


def declared_symbols():
    text = open(os.path.join(ROOT, "include", "neofiz.h")).read()
    text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
    return sorted(set(re.findall(r"\b(nf_[a-z_]+)\s*\(", text)))


@pytest.fixture(scope="module")
def library():
    from neofiz_gb300 import build
    return build.build()


def test_header_declares_the_solver_surface():
    names = declared_symbols()
    for required in ("nf_create", "nf_destroy", "nf_step", "nf_read_field", "nf_set_contact",
                     "nf_set_rigid_wall", "nf_set_damage", "nf_set_erosion", "nf_audits",
                     "nf_material_point_update", "nf_run_until"):
        assert required in names


def test_library_exports_every_declared_symbol(library):
    """Loaded in a subprocess so that no CUDA state lingers in the test process."""
    code = ("import ctypes,sys; lib=ctypes.CDLL(sys.argv[1]); "
            "missing=[n for n in sys.argv[2:] if not hasattr(lib, n)]; "
            "print(' '.join(missing)); sys.exit(1 if missing else 0)")
    r = subprocess.run([sys.executable, "-c", code, library, *declared_symbols()],
                       capture_output=True, text=True)
    assert r.returncode == 0, f"missing exports: {r.stdout} {r.stderr}"


DEVICE_ONLY = {"nf_device_count", "nf_material_point_update_static", "nf_device_fp64_rate"}
# the device film has no CPU counterpart (it captures device memory)
FILM = {"nf_film_create", "nf_film_destroy", "nf_film_capture", "nf_film_frames",
        "nf_film_read", "nf_film_clear", "nf_film_last_error"}


def test_abi_binding_covers_the_header():
    from neofiz_gb300 import _abi
    declared = set(declared_symbols()) - DEVICE_ONLY - FILM
    assert declared == set(_abi.ENTRY_POINTS)
    assert FILM == {"nf_" + name for name in _abi._FILM_PROTOS}


def test_oracle_exports_the_same_surface():
    from oracle import oracle
    lib = ctypes.CDLL(oracle.build())
    for name in declared_symbols():
        if name in DEVICE_ONLY or name in FILM:
            continue
        assert hasattr(lib, "nfo_" + name[3:]), name


def test_struct_layouts_match_the_header():
    """Sizes of the ctypes mirrors against a C compile of the header."""
    from neofiz_gb300 import _abi
    src = ("#include <stdio.h>\n#include \"neofiz.h\"\nint main(){printf(\"%zu %zu %zu %zu %zu "
           "%zu %zu %zu %zu %zu %zu %zu %zu\\n\", sizeof(nf_mesh), sizeof(nf_material), "
           "sizeof(nf_state), sizeof(nf_audit), sizeof(nf_wall_info), sizeof(nf_contact_info), "
           "sizeof(nf_measure), sizeof(nf_damage_points), sizeof(nf_batch_mesh), "
           "sizeof(nf_batch_instance), sizeof(nf_batch_config), sizeof(nf_batch_progress), "
           "sizeof(nf_film_info)); "
           "return 0;}\n")
    import tempfile
    with tempfile.TemporaryDirectory() as d:
        c = os.path.join(d, "s.c")
        open(c, "w").write(src)
        exe = os.path.join(d, "s")
        subprocess.check_call(["gcc", "-I", os.path.join(ROOT, "include"), c, "-o", exe])
        sizes = [int(x) for x in subprocess.check_output([exe]).split()]
    mine = [ctypes.sizeof(t) for t in (_abi.Mesh, _abi.MaterialC, _abi.State, _abi.Audit,
                                        _abi.WallInfo, _abi.ContactInfo, _abi.Measure,
                                        _abi.DamagePoints, _abi.BatchMesh, _abi.BatchInstance,
                                        _abi.BatchConfig, _abi.BatchProgress, _abi.FilmInfo)]
    assert sizes == mine


def test_product_fails_loudly_without_a_device(library):
    """With no CUDA device the product raises instead of falling back to anything."""
    code = ("import sys; sys.path.insert(0, sys.argv[1]);\n"
            "from neofiz_gb300 import _native\n"
            "try:\n    _native.api()\nexcept _native.NativeUnavailable as e:\n"
            "    print('unavailable:', e); sys.exit(0)\n"
            "print('device present'); sys.exit(0)\n")
    r = subprocess.run([sys.executable, "-c", code, ROOT], capture_output=True, text=True)
    assert r.returncode == 0
    assert ("unavailable" in r.stdout) or ("device present" in r.stdout)
