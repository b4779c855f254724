"""The seeded Zel'dovich IC generator and the reference's file format."""
import math
import os
import tempfile

import numpy as np

from cuco_gb300 import ics


def test_deterministic_and_in_box():
    a = ics.zeldovich(16, 50.0, 49.0, seed=3)
    b = ics.zeldovich(16, 50.0, 49.0, seed=3)
    c = ics.zeldovich(16, 50.0, 49.0, seed=4)
    assert np.array_equal(a.pos, b.pos) and np.array_equal(a.vel, b.vel)
    assert not np.array_equal(a.pos, c.pos)
    assert a.pos.dtype == np.float32 and a.pos.shape == (16 ** 3, 3)
    assert (a.pos >= 0).all() and (a.pos < np.float32(a.boxsize)).all()


def test_mass_matches_omega_as_check_omega():
    ic = ics.zeldovich(16, 50.0, 49.0, seed=1)
    # init.c:52: omega = sum(m) / L^3 / (3 H^2 / (8 pi G))
    omega = ic.n * np.float32(ic.mass) / ic.boxsize ** 3 / (
        3 * ics.HUBBLE_INTERNAL ** 2 / (8 * math.pi * ics.G_INTERNAL))
    assert abs(omega - 0.3) < 1e-6


def test_zeldovich_velocity_displacement_relation():
    """v_pec = a H f D psi: velocity is parallel to the displacement."""
    ic = ics.zeldovich(16, 50.0, 49.0, seed=2)
    n, L = 16, ic.boxsize
    q = (np.arange(n) + 0.5) * (L / n)
    Q = np.stack(np.meshgrid(q, q, q, indexing="ij"), -1).reshape(-1, 3)
    disp = ic.pos.astype(np.float64) - Q
    disp -= L * np.round(disp / L)
    D, f = ic.cosmology.growth(ic.a)
    H = ics.HUBBLE_INTERNAL * ic.cosmology.E(ic.a)
    vexp = ic.a * H * f * disp / math.sqrt(ic.a)
    assert np.allclose(ic.vel, vexp, rtol=1e-3, atol=1e-3 * np.abs(vexp).max())


def test_growth_factor_limits():
    c = ics.Cosmology()
    d1, f1 = c.growth(1.0)
    assert abs(d1 - 1.0) < 1e-9
    d, f = c.growth(0.02)
    assert abs(d / 0.02 - 1.28) < 0.05      # matter era: D ~ a (normalised to D(1) = 0.78 a)
    assert abs(f - 1.0) < 1e-3              # f -> 1 in matter domination
    assert abs(f1 - 0.3 ** 0.55) < 0.02     # f ~ Omega_m^0.55 today


def test_sigma8_normalisation():
    c = ics.Cosmology()
    A = c.power_amplitude()
    from scipy.integrate import quad

    def integrand(lnk):
        k = math.exp(lnk)
        x = 8.0 * k
        w = 3 * (math.sin(x) - x * math.cos(x)) / x ** 3
        return k ** 3 * A * k ** c.ns * float(c.transfer_bbks(k)) ** 2 * w * w / (2 * math.pi ** 2)
    s2 = quad(integrand, math.log(1e-4), math.log(1e2), limit=400)[0]
    assert abs(math.sqrt(s2) - 0.8) < 1e-3


def test_file_roundtrip():
    ic = ics.zeldovich(8, 20.0, 49.0, seed=5)
    with tempfile.TemporaryDirectory() as td:
        p = os.path.join(td, "ic.cuco")
        ics.write_cuco(p, ic)
        assert os.path.getsize(p) == 32 + 60 * ic.n
        hdr, parts = ics.read_cuco(p)
    assert int(hdr["NumPart"]) == ic.n
    assert np.float32(hdr["BoxSize"]) == np.float32(ic.boxsize)
    assert np.array_equal(parts["Pos"], ic.pos) and np.array_equal(parts["Vel"], ic.vel)
    assert np.all(parts["Mass"] == np.float32(ic.mass))
