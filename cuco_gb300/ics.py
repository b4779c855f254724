"""Seeded Zel'dovich initial conditions and the reference's particle file format.

The workloads are synthetic: a Gaussian random field with
P(k) ~ k^ns T_BBKS(k)^2 (Bardeen, Bond, Kaiser & Szalay 1986, eq. G3, with
Gamma = Omega_m h), normalised to sigma_8 with a top-hat window at z = 0 and
scaled to the start time by the linear growth factor, displaces particles from
a regular lattice (Zel'dovich 1970).  White noise comes from numpy's Philox
counter-based generator keyed by the seed.

Units are the reference's (begrun.c:33-35, 65-78): length kpc/h, mass
1e10 Msun/h, velocity km/s.  Velocities are written in the reference's file
convention u = v_pec / sqrt(a); init.c:30 multiplies them by a^{3/2} to get the
canonical momentum a^2 dx/dt.  The particle mass is chosen so that the
reference's check_omega (init.c:41-58) passes.

File format (read_ic.c:19-33, io.c:22-34): a 32-byte HEADER
{int NumPart; float Mass, Time, Redshift, BoxSize, Omega0, OmegaLambda,
HubbleParam} followed by NumPart 60-byte PARTICLE records
{float Pos[3], Mass, Vel[3], GravAccel[3], GravPM[3]; int Ti_endstep, Ti_begstep}
(allvars.h:35-57), native byte order.
"""
from __future__ import annotations

import math
from dataclasses import dataclass

import numpy as np

# unit system of the reference (begrun.c:33-35,67-70; allvars.h:15-18)
UNIT_LENGTH_M = 3.085678e19
UNIT_MASS_KG = 1.98892e40
UNIT_VELOCITY_MS = 1e3
UNIT_TIME_S = UNIT_LENGTH_M / UNIT_VELOCITY_MS
GRAVITY_SI = 6.673e-11
HUBBLE_SI = 3.2407789e-18
G_INTERNAL = GRAVITY_SI / UNIT_LENGTH_M ** 3 * UNIT_MASS_KG * UNIT_TIME_S ** 2
HUBBLE_INTERNAL = HUBBLE_SI * UNIT_TIME_S

HEADER_DTYPE = np.dtype([
    ("NumPart", "<i4"), ("Mass", "<f4"), ("Time", "<f4"), ("Redshift", "<f4"),
    ("BoxSize", "<f4"), ("Omega0", "<f4"), ("OmegaLambda", "<f4"), ("HubbleParam", "<f4"),
])
PARTICLE_DTYPE = np.dtype([
    ("Pos", "<f4", 3), ("Mass", "<f4"), ("Vel", "<f4", 3), ("GravAccel", "<f4", 3),
    ("GravPM", "<f4", 3), ("Ti_endstep", "<i4"), ("Ti_begstep", "<i4"),
])
assert HEADER_DTYPE.itemsize == 32 and PARTICLE_DTYPE.itemsize == 60


@dataclass
class Cosmology:
    omega0: float = 0.3
    omega_lambda: float = 0.7
    hubble_param: float = 0.7
    sigma8: float = 0.8
    ns: float = 0.96

    def E(self, a):
        ok = 1.0 - self.omega0 - self.omega_lambda
        return np.sqrt(self.omega0 / a ** 3 + ok / a ** 2 + self.omega_lambda)

    def growth(self, a):
        """Linear growth D(a) normalised to D(1) = 1, and f = dlnD/dlna.

        D ~ E(a) int_0^a da' / (a' E(a'))^3 (Heath 1977), valid for matter plus
        cosmological constant plus curvature."""
        from scipy.integrate import quad

        def integral(x):
            return quad(lambda s: 1.0 / (s * self.E(s)) ** 3, 0.0, x, epsabs=0, epsrel=1e-11,
                        limit=200)[0]
        ia, i1 = integral(a), integral(1.0)
        d = self.E(a) * ia / (self.E(1.0) * i1)
        ok = 1.0 - self.omega0 - self.omega_lambda
        dlnE = -(3 * self.omega0 / a ** 3 + 2 * ok / a ** 2) / (2 * self.E(a) ** 2)
        f = dlnE + 1.0 / (a ** 2 * self.E(a) ** 3 * ia)
        return float(d), float(f)

    def transfer_bbks(self, k_hmpc):
        gamma = self.omega0 * self.hubble_param
        q = np.asarray(k_hmpc, dtype=np.float64) / gamma
        q = np.where(q == 0, 1e-30, q)
        return (np.log(1 + 2.34 * q) / (2.34 * q)
                * (1 + 3.89 * q + (16.1 * q) ** 2 + (5.46 * q) ** 3 + (6.71 * q) ** 4) ** -0.25)

    def power_amplitude(self):
        """Amplitude A of P(k) = A k^ns T^2 (k in h/Mpc, P in (Mpc/h)^3) giving sigma_8."""
        from scipy.integrate import quad
        R = 8.0

        def integrand(lnk):
            k = math.exp(lnk)
            x = k * R
            w = 3.0 * (math.sin(x) - x * math.cos(x)) / x ** 3
            return k ** 3 * k ** self.ns * float(self.transfer_bbks(k)) ** 2 * w * w / (2 * math.pi ** 2)
        s2 = quad(integrand, math.log(1e-5), math.log(1e3), limit=500, epsrel=1e-10)[0]
        return self.sigma8 ** 2 / s2


def particle_mass(n_total: int, boxsize_kpc: float, omega0: float) -> float:
    """Equal particle mass so that sum(m) / L^3 = Omega0 * rho_crit (init.c:52)."""
    rho_crit = 3 * HUBBLE_INTERNAL ** 2 / (8 * math.pi * G_INTERNAL)
    return omega0 * rho_crit * boxsize_kpc ** 3 / n_total


@dataclass
class InitialConditions:
    pos: np.ndarray      # (N, 3) float32, kpc/h, in [0, L)
    vel: np.ndarray      # (N, 3) float32, km/s, file convention v_pec / sqrt(a)
    mass: float
    boxsize: float       # kpc/h
    a: float
    cosmology: Cosmology

    @property
    def n(self) -> int:
        return self.pos.shape[0]

    def canonical_velocity(self) -> np.ndarray:
        """Velocity in the integrator's variable a^2 dx/dt (init.c:30)."""
        return (self.vel.astype(np.float64) * (math.sqrt(self.a) * self.a)).astype(np.float32)


def zeldovich(n_side: int, boxsize_mpc: float, z_init: float, seed: int,
              cosmo: Cosmology | None = None) -> InitialConditions:
    """n_side^3 particles in a periodic box of boxsize_mpc Mpc/h at redshift z_init."""
    cosmo = cosmo or Cosmology()
    L = boxsize_mpc * 1000.0                      # kpc/h
    a = 1.0 / (1.0 + z_init)
    n = n_side
    rng = np.random.Generator(np.random.Philox(key=seed))
    noise = rng.standard_normal((n, n, n))
    wk = np.fft.rfftn(noise)
    kf = 2 * math.pi / boxsize_mpc                 # h/Mpc
    kx = np.fft.fftfreq(n, d=1.0 / n) * kf
    kz = np.fft.rfftfreq(n, d=1.0 / n) * kf
    KX, KY, KZ = np.meshgrid(kx, kx, kz, indexing="ij")
    k2 = KX ** 2 + KY ** 2 + KZ ** 2
    k = np.sqrt(k2)
    A = cosmo.power_amplitude()
    pk = np.where(k > 0, A * np.where(k > 0, k, 1.0) ** cosmo.ns * cosmo.transfer_bbks(k) ** 2, 0.0)
    cell = boxsize_mpc / n                         # Mpc/h
    delta_k = wk * np.sqrt(pk / cell ** 3)
    nyq = n // 2
    idx = np.fft.fftfreq(n, d=1.0 / n)
    zero = (np.abs(idx)[:, None, None] == nyq) | (np.abs(idx)[None, :, None] == nyq)
    zero = zero | (np.fft.rfftfreq(n, d=1.0 / n)[None, None, :] == nyq)
    delta_k = np.where(zero | (k2 == 0), 0.0, delta_k)
    inv_k2 = np.where(k2 > 0, 1.0 / np.where(k2 > 0, k2, 1.0), 0.0)
    D, f = cosmo.growth(a)
    disp = np.empty((n, n, n, 3), dtype=np.float64)
    for d, K in enumerate((KX, KY, KZ)):
        psi_k = 1j * K * inv_k2 * delta_k           # Mpc/h at z = 0
        disp[..., d] = np.fft.irfftn(psi_k, s=(n, n, n), axes=(0, 1, 2)) * 1000.0 * D  # kpc/h at a
    q = (np.arange(n) + 0.5) * (L / n)
    Q = np.stack(np.meshgrid(q, q, q, indexing="ij"), axis=-1)
    pos = np.mod(Q + disp, L).reshape(-1, 3)
    pos = pos.astype(np.float32)
    pos[pos >= np.float32(L)] = 0.0
    hubble_a = HUBBLE_INTERNAL * cosmo.E(a)
    vpec = a * hubble_a * f * disp.reshape(-1, 3)  # a dx/dt, km/s
    vel = (vpec / math.sqrt(a)).astype(np.float32)
    mass = particle_mass(n ** 3, L, cosmo.omega0)
    return InitialConditions(pos=pos, vel=vel, mass=mass, boxsize=L, a=a, cosmology=cosmo)


def write_cuco(path: str, ic: InitialConditions, time: float | None = None) -> None:
    """Write HEADER + PARTICLE[] as read_ic.c:19-33 reads it."""
    hdr = np.zeros(1, dtype=HEADER_DTYPE)
    a = ic.a if time is None else time
    hdr["NumPart"] = ic.n
    hdr["Mass"] = ic.mass
    hdr["Time"] = a
    hdr["Redshift"] = 1.0 / a - 1.0
    hdr["BoxSize"] = ic.boxsize
    hdr["Omega0"] = ic.cosmology.omega0
    hdr["OmegaLambda"] = ic.cosmology.omega_lambda
    hdr["HubbleParam"] = ic.cosmology.hubble_param
    parts = np.zeros(ic.n, dtype=PARTICLE_DTYPE)
    parts["Pos"] = ic.pos
    parts["Mass"] = ic.mass
    parts["Vel"] = ic.vel
    with open(path, "wb") as fh:
        fh.write(hdr.tobytes())
        fh.write(parts.tobytes())


def read_cuco(path: str):
    """Read a snapshot or IC file: returns (header record, particle records)."""
    raw = np.fromfile(path, dtype=np.uint8)
    hdr = raw[:32].view(HEADER_DTYPE)[0]
    n = int(hdr["NumPart"])
    parts = raw[32:32 + 60 * n].view(PARTICLE_DTYPE)
    return hdr, parts
