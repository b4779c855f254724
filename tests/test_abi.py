"""The C ABI: the library loads without a GPU, exports every function the
public headers declare, and its structs have the reference's layout."""
import ctypes
import os
import re
import subprocess
import tempfile

import numpy as np
import pytest

import oracle
from cuco_gb300 import _native

ROOT = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
HEADERS = [os.path.join(ROOT, "include", f) for f in ("cuco_gb300.h", "cuco_allvars.h")]


def declared_functions():
    names = set()
    for h in HEADERS:
        text = open(h).read()
        text = re.sub(r"/\*.*?\*/", "", text, flags=re.S)
        for m in re.finditer(r"^\s*(?:const\s+)?[A-Za-z_][\w\s\*]*?\b([A-Za-z_]\w*)\s*\(", text, flags=re.M):
            name = m.group(1)
            if name not in ("if", "while", "for", "sizeof", "defined"):
                names.add(name)
    return names


@pytest.fixture(scope="module")
def lib():
    from cuco_gb300 import build
    build.build()
    return _native.load()


def test_library_exports_every_declared_function(lib):
    names = declared_functions()
    assert len(names) >= 59
    missing = [n for n in sorted(names) if not hasattr(lib, n)]
    assert not missing, missing
    # and the ctypes binding covers them all
    assert names <= set(_native.SIGNATURES), names - set(_native.SIGNATURES)


def test_reference_globals_are_exported(lib):
    for g in ("P", "NumPart", "All", "header", "DriftTable", "GravKickTable", "sorter", "dOldPos",
              "dSortedPos", "dGravAccel", "dGridParticleHash", "dGridParticleIndex", "dCellStart",
              "dCellEnd", "numParticles", "numGridCells", "hPos", "hGravAccel"):
        ctypes.c_void_p.in_dll(lib, g)


def test_struct_sizes():
    assert ctypes.sizeof(_native.Particle) == 60
    assert ctypes.sizeof(_native.Header) == 32
    assert ctypes.sizeof(_native.SimParam) == 4 * 1009
    assert ctypes.sizeof(_native.SoftParam) == 12


@pytest.mark.skipif(not oracle.reference_available(), reason="reference sources not present")
def test_layout_matches_reference_build():
    ref = oracle.Reference(32)
    out = (ctypes.c_long * 16)()
    ref.lib.cref_layout(out)
    A = _native.All
    mine = [ctypes.sizeof(A), A.G.offset, A.Hubble.offset, A.Time.offset, A.Timebase_interval.offset,
            A.Ti_Current.offset, A.PM_Ti_endstep.offset, A.Asmth.offset, A.ForceSoftening.offset,
            A.OutputListTimes.offset, A.InitCondFile.offset, ctypes.sizeof(_native.Particle),
            ctypes.sizeof(_native.Header), _native.Particle.GravPM.offset,
            _native.Particle.Ti_endstep.offset, A.SofteningTable.offset]
    assert list(out) == mine


def test_header_compiles_as_c_with_reference_layout():
    src = r'''
#include <stddef.h>
#include "cuco_gb300.h"
_Static_assert(sizeof(PARTICLE) == 60, "PARTICLE");
_Static_assert(sizeof(HEADER) == 32, "HEADER");
_Static_assert(offsetof(ALL, Timebase_interval) == %d, "ALL");
_Static_assert(sizeof(ALL) == %d, "ALL size");
int main(void) { return 0; }
''' % (_native.All.Timebase_interval.offset, ctypes.sizeof(_native.All))
    with tempfile.TemporaryDirectory() as td:
        f = os.path.join(td, "t.c")
        open(f, "w").write(src)
        r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", os.path.join(ROOT, "include"),
                            f, "-o", os.path.join(td, "t")], capture_output=True, text=True)
        assert r.returncode == 0, r.stderr


def test_dropin_drift_tables_host(lib):
    """init_drift_table / get_drift_factor / get_gravkick_factor are host code:
    FP64 tables with driftfac.c's interpolation, equal to the oracle's."""
    from cuco_gb300._native import All
    f32 = lambda v: float(np.float32(v))  # noqa: E731
    al = All.in_dll(lib, "All")
    al.Omega0, al.OmegaLambda, al.Hubble = 0.3, 0.7, 0.1
    al.TimeBegin, al.TimeMax = 0.02, 1.0
    al.Timebase_interval = (np.log(1.0) - np.log(np.float32(0.02))) / (1 << 28)
    lib.init_drift_table()
    port = oracle.Port()
    d, k = port.drift_tables(f32(0.02), 1.0, f32(0.3), f32(0.7), f32(0.1))
    l0 = np.log(f32(0.02))
    for t0, t1 in [(0, 1 << 20), (1 << 20, 1 << 22), (7, 1 << 28)]:
        assert lib.get_drift_factor(t0, t1) == port.table_factor(d, l0, 0.0, al.Timebase_interval, t0, t1)
        assert lib.get_gravkick_factor(t0, t1) == port.table_factor(k, l0, 0.0, al.Timebase_interval, t0, t1)
    tab = (ctypes.c_float * 1000).in_dll(lib, "DriftTable")
    assert np.array_equal(np.array(tab[:], dtype=np.float32), d.astype(np.float32))
    a = 0.5
    assert lib.drift_integ(a, None) == pytest.approx(1 / (0.1 * np.sqrt(f32(0.3) / a ** 3 + f32(0.7)) * a ** 3), rel=1e-7)


def test_host_only_entry_points(lib):
    """FP64 integrals run on the host: no device needed."""
    d, k = ctypes.c_double(), ctypes.c_double()
    assert lib.cuco_cosmo_factors(0.02, 1.0, 0.3, 0.7, 0.1, ctypes.byref(d), ctypes.byref(k)) == 0
    port = oracle.Port()
    dt, kt = port.drift_tables(0.02, 1.0, 0.3, 0.7, 0.1, 10)
    assert d.value == pytest.approx(dt[-1], rel=1e-12)
    assert k.value == pytest.approx(kt[-1], rel=1e-12)
    assert lib.cuco_cosmo_factors(-1.0, 1.0, 0.3, 0.7, 0.1, ctypes.byref(d), ctypes.byref(k)) == 1
    assert b"positive" in lib.cuco_last_error()
    assert lib.cuco_version().startswith(b"cuco_gb300")


def test_reference_style_hosts_link(lib, tmp_path):
    """Hosts that keep the reference's calls link against the headers and the
    library alone: the C++ host with gravlist.cpp's `RadixSort` use
    (tests/gravlist_host.cpp, run on the GPU by test_gpu_radixsort_host.py),
    and a C host that defines its own globals as allvars.c does and calls the
    reference-named drop-in functions in begrun's and run.c's order.  Nothing
    is run here."""
    lib_dir = os.path.dirname(_native.LIB_PATH)
    inc = os.path.join(ROOT, "include")
    link = ["-L", lib_dir, "-lcuco_gb300", "-Wl,-rpath," + lib_dir]
    r = subprocess.run(["g++", "-O1", "-std=c++11", "-Wall", "-Werror", "-I", inc,
                        os.path.join(ROOT, "tests", "gravlist_host.cpp"), *link,
                        "-o", str(tmp_path / "gravlist_host")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
    src = tmp_path / "run_loop.c"
    src.write_text(r'''
#include "cuco_gb300.h"
/* the host's own globals, as allvars.c:7-10 defines them */
unsigned int NumPart;
PARTICLE *P;
HEADER header;
ALL All;
int main(int argc, char **argv) {
    if (argc < 2) return 0;           /* linked, not run */
    read_ic(argv[1]);
    init_drift_table();
    long_range_init();
    linklist_init();
    compute_accelerations();
    move_particles(All.Ti_Current, All.Ti_Current + 1);
    advance_and_find_timesteps();
    savepositions(0);
    return 0;
}
''')
    r = subprocess.run(["gcc", "-std=c11", "-Wall", "-Werror", "-I", inc, str(src), *link,
                        "-o", str(tmp_path / "run_loop")], capture_output=True, text=True)
    assert r.returncode == 0, r.stderr
