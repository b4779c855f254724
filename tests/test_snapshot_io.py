"""The reference's IC/snapshot file format, HEADER (32 bytes) then
PARTICLE[NumPart] (60 bytes each) raw (read_ic.c:9-45, io.c:9-40):

* read_ic / savepositions, the reference-named host functions (no GPU): an IC
  file read into the globals and written back as snapshot <num> is the same
  bytes, apart from the redshift that io.c:28 recomputes from All.Time in
  float;
* a serving job's output snapshot (host code): the same format, read back by
  read_ic; its drift to the output time as predict.c computes it;
* cuco_box_load_snapshot / cuco_box_save_snapshot (GPU): a file loaded into a
  box and saved again keeps Pos, Vel and Mass bit for bit and carries the
  box's last forces in GravAccel/GravPM."""
import ctypes
import os

import numpy as np
import pytest

from cuco_gb300 import Box, BoxConfig, _native, ics
from cuco_gb300._native import All, Header
from cuco_gb300.engine import MODE_FIXED
from cuco_gb300.ics import read_cuco, write_cuco


def _ic(n_side=8, seed=3):
    return ics.zeldovich(n_side, 20.0, 49.0, seed)


def test_read_ic_and_savepositions_round_trip(tmp_path):
    lib = _native.load()
    ic = _ic()
    src = tmp_path / "ic.cuco"
    write_cuco(str(src), ic)
    lib.read_ic(str(src).encode())
    n = ctypes.c_uint.in_dll(lib, "NumPart").value
    assert n == ic.n
    hdr = Header.in_dll(lib, "header")
    al = All.in_dll(lib, "All")
    assert al.NumPart == ic.n and al.BoxSize == np.float32(ic.boxsize) and al.Mass == np.float32(ic.mass)
    assert hdr.Time == np.float32(ic.a)
    # the records are the file's
    p = ctypes.c_void_p.in_dll(lib, "P").value
    recs = np.frombuffer((ctypes.c_uint8 * (60 * n)).from_address(p), dtype=np.uint8).copy()
    raw = np.fromfile(src, dtype=np.uint8)
    assert np.array_equal(recs, raw[32:])
    # savepositions(3) into <OutputDir>/<SnapshotFileBase>_3.cuco
    al.OutputDir = str(tmp_path).encode()
    al.SnapshotFileBase = b"snap"
    al.Time = hdr.Time
    lib.savepositions(3)
    out = np.fromfile(tmp_path / "snap_3.cuco", dtype=np.uint8)
    assert out.size == raw.size
    assert np.array_equal(out[32:], raw[32:])
    h_in, h_out = raw[:32].view(np.float32), out[:32].view(np.float32)
    same = [0, 1, 2, 4, 5, 6, 7]  # all but the redshift (index 3)
    assert np.array_equal(h_in[same], h_out[same])
    assert h_out[3] == np.float32(np.float32(1) / np.float32(hdr.Time) - np.float32(1))


def test_serving_output_snapshot_is_the_reference_format(tmp_path):
    """A serving job's output snapshot (host code, no GPU): the reference's
    HEADER + PARTICLE[] with the drifted positions, the velocities and both
    forces; the drop-in's read_ic reads it as the reference would."""
    from cuco_gb300.serve import Job, output_positions, write_snapshot
    ic = _ic()
    cfg = BoxConfig(n=ic.n, pm_grid=16, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL, softening=1.0)
    vel = ic.canonical_velocity()
    job = Job(7, cfg, ic.pos, vel, ic.a, 10, omega0=0.25, omega_lambda=0.75, hubble_param=0.68)
    rng = np.random.default_rng(5)
    acc_pp = rng.normal(size=(ic.n, 3)).astype(np.float32)
    acc_pm = rng.normal(size=(ic.n, 3)).astype(np.float32)
    # a drift large enough that some particles cross the box edge
    pos = output_positions(ic.pos, vel, 0.02 * ic.boxsize / float(np.abs(vel).max()), ic.boxsize)
    assert pos.dtype == np.float32 and pos.min() >= 0 and pos.max() < np.float32(ic.boxsize)
    path = tmp_path / "job7_out0.cuco"
    write_snapshot(str(path), job, 0.25, pos, vel, acc_pp, acc_pm)
    hdr, parts = read_cuco(str(path))
    assert hdr["NumPart"] == ic.n and hdr["Time"] == np.float32(0.25) and hdr["Redshift"] == np.float32(3.0)
    assert hdr["BoxSize"] == np.float32(ic.boxsize) and hdr["Mass"] == np.float32(ic.mass)
    assert (hdr["Omega0"], hdr["OmegaLambda"], hdr["HubbleParam"]) == (np.float32(0.25), np.float32(0.75),
                                                                        np.float32(0.68))
    for name, want in (("Pos", pos), ("Vel", vel), ("GravAccel", acc_pp), ("GravPM", acc_pm)):
        assert np.array_equal(parts[name], want), name
    assert np.all(parts["Mass"] == np.float32(ic.mass))
    lib = _native.load()
    lib.read_ic(str(path).encode())
    n = ctypes.c_uint.in_dll(lib, "NumPart").value
    assert n == ic.n
    p = ctypes.c_void_p.in_dll(lib, "P").value
    recs = np.frombuffer((ctypes.c_uint8 * (60 * n)).from_address(p), dtype=np.uint8).copy()
    assert np.array_equal(recs, np.fromfile(path, dtype=np.uint8)[32:])


def test_output_positions_follow_predict_c():
    """The drift to an output time and the box wrapping, element by element
    as predict.c:19,34-38 computes them (a float position plus a float
    velocity times a double drift, in double, stored as float; then L added
    or subtracted in double while outside [0, L))."""
    from cuco_gb300.serve import output_positions
    rng = np.random.default_rng(8)
    L = 20000.0
    pos = rng.uniform(0, L, (500, 3)).astype(np.float32)
    pos[:5] = [[0.0, L * (1 - 2 ** -20), 1.0]] * 5
    vel = rng.normal(0, 300, (500, 3)).astype(np.float32)
    drift = 3.7
    got = output_positions(pos, vel, drift, L)
    want = np.empty_like(pos)
    for i in range(pos.shape[0]):
        for j in range(3):
            x = np.float32(float(pos[i, j]) + float(vel[i, j]) * drift)
            while x < 0:
                x = np.float32(float(x) + L)
            while x >= L:
                x = np.float32(float(x) - L)
            want[i, j] = x
    assert np.array_equal(got, want)


@pytest.mark.gpu
@pytest.mark.parametrize("mode", [0, MODE_FIXED])
def test_box_snapshot_load_save(tmp_path, mode):
    ic = _ic(16, 5)
    src = tmp_path / "ic.cuco"
    write_cuco(str(src), ic)
    soft = 2.8 * 0.03 * ic.boxsize / 16
    box = Box(BoxConfig(n=ic.n, pm_grid=32, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                        softening=soft, mode=mode))
    hdr = box.load_snapshot(str(src), initial_conditions=True)
    assert hdr.NumPart == ic.n and hdr.Time == np.float32(ic.a)
    pos, vel, _, _ = box.get_state()
    # init.c:30: IC velocities are scaled by a^(3/2) into the integrator's variable
    scale = np.float32(np.sqrt(np.float64(hdr.Time)) * np.float64(hdr.Time))
    assert np.array_equal(vel, (ic.vel * scale).astype(np.float32))
    if mode == 0:
        assert np.array_equal(pos, ic.pos)
    else:  # fixed point rounds positions to L / 2^32
        assert np.abs(pos - ic.pos).max() <= 1e-6 * ic.boxsize
    box.forces()
    _, _, app, apm = box.get_state()
    snap = tmp_path / "snap.cuco"
    box.save_snapshot(str(snap), hdr)
    h2, parts = read_cuco(str(snap))
    assert int(h2["NumPart"]) == ic.n and h2["Time"] == hdr.Time and h2["BoxSize"] == hdr.BoxSize
    assert np.array_equal(parts["Pos"], pos) and np.array_equal(parts["Vel"], vel)
    assert np.all(parts["Mass"] == np.float32(ic.mass))
    assert np.array_equal(parts["GravAccel"], app) and np.array_equal(parts["GravPM"], apm)
    assert not parts["Ti_endstep"].any() and not parts["Ti_begstep"].any()
    # a snapshot loads back as stored (no velocity scaling) and saves to the same bytes
    box2 = Box(BoxConfig(n=ic.n, pm_grid=32, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                         softening=soft, mode=mode))
    box2.load_snapshot(str(snap), initial_conditions=False)
    box2.forces()
    snap2 = tmp_path / "snap2.cuco"
    box2.save_snapshot(str(snap2), hdr)
    if mode == 0:
        assert np.array_equal(np.fromfile(snap, dtype=np.uint8), np.fromfile(snap2, dtype=np.uint8))
    else:  # positions pass through the 2^-32 grid again; the state is unchanged
        _, p2 = read_cuco(str(snap2))
        assert np.array_equal(p2["Pos"], parts["Pos"]) and np.array_equal(p2["Vel"], parts["Vel"])
    # a file for another particle count is refused
    box3 = Box(BoxConfig(n=ic.n + 1, pm_grid=32, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL,
                         softening=soft, mode=mode))
    with pytest.raises(Exception):
        box3.load_snapshot(str(snap))
    for b in (box, box2, box3):
        b.close()
    os.remove(snap)


def test_read_ic_exits_on_a_truncated_file(tmp_path):
    """read_ic.c:12-15 exits with a message on a missing file; the library's
    read_ic does the same for a file that ends before its particles."""
    import subprocess
    import sys
    ic = _ic()
    src = tmp_path / "ic.cuco"
    write_cuco(str(src), ic)
    raw = np.fromfile(src, dtype=np.uint8)
    (tmp_path / "short.cuco").write_bytes(raw[: 32 + 60 * (ic.n // 2)].tobytes())
    root = os.path.dirname(os.path.dirname(os.path.abspath(__file__)))
    for name in ("short.cuco", "missing.cuco"):
        code = ("import sys; sys.path.insert(0, %r); from cuco_gb300 import _native; "
                "_native.load().read_ic(%r)" % (root, str(tmp_path / name).encode()))
        r = subprocess.run([sys.executable, "-c", code], capture_output=True, text=True, timeout=120)
        assert r.returncode == 1, (r.returncode, r.stdout, r.stderr)
        assert "initial condition file" in r.stdout.lower()


@pytest.mark.gpu
def test_invalid_state_and_files_are_refused(tmp_path):
    """An invalid IC file (truncated) and a state with a NaN injected into the
    host-side copy are refused with an error status; the box keeps working."""
    ic = _ic(16, 9)
    soft = 2.8 * 0.03 * ic.boxsize / 16
    box = Box(BoxConfig(n=ic.n, pm_grid=32, boxsize=ic.boxsize, mass=ic.mass, G=ics.G_INTERNAL, softening=soft))
    src = tmp_path / "ic.cuco"
    write_cuco(str(src), ic)
    raw = np.fromfile(src, dtype=np.uint8)
    (tmp_path / "short.cuco").write_bytes(raw[:-60].tobytes())
    with pytest.raises(Exception, match="ends before"):
        box.load_snapshot(str(tmp_path / "short.cuco"))
    pos = ic.pos.copy()
    pos[123, 2] = np.nan
    with pytest.raises(Exception, match="not finite"):
        box.set_state(pos, ic.canonical_velocity())
    vel = ic.canonical_velocity().copy()
    vel[5, 0] = np.inf
    with pytest.raises(Exception, match="not finite"):
        box.set_state(ic.pos, vel)
    box.set_state(ic.pos, ic.canonical_velocity())
    box.forces()
    _, _, app, apm = box.get_state()
    assert np.isfinite(app).all() and np.isfinite(apm).all()
    box.close()
