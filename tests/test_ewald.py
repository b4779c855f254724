"""The FP64 Ewald oracle (oracle/ewald.c) checked on its own, before anything is
measured against it:

* the split parameter alpha only moves work between the real and Fourier
  sums: two values give the same forces to ~1e-10;
* a perfect cubic lattice feels no force (symmetry, and the neutralising
  background);
* a close pair in a large box feels Newton plus the cubic-lattice background
  term, a = G m [d/|d|^3 - (4 pi/3) d/L^3] (the image lattice's tidal field
  vanishes at first order by cubic symmetry), to the O((d/L)^5) remainder;
* inside the softening length the pair force is the reference's spline
  (gravlist.cpp:307-316) plus the same background term.
"""
import numpy as np
import pytest

from conftest import rms_rel


def test_alpha_independence(port):
    rng = np.random.default_rng(11)
    L, n = 1000.0, 3000
    src = rng.uniform(0, L, (n, 3))
    # clustered part so that near and far pairs both matter
    src[:1000] = np.mod(src[0] + rng.normal(0, 20.0, (1000, 3)), L)
    tg = src[rng.choice(n, 200, replace=False)]
    a1 = port.ewald(src, 1.0, 1.0, L, 1.0, tg, 8, alpha_l=12.0)
    a2 = port.ewald(src, 1.0, 1.0, L, 1.0, tg, 8, alpha_l=20.0)
    a3 = port.ewald(src, 1.0, 1.0, L, 1.0, tg, 8)  # automatic choice
    assert rms_rel(a1, a2) < 1e-10
    assert rms_rel(a3, a2) < 1e-10


def test_lattice_feels_no_force(port):
    L, k = 100.0, 8
    g = (np.arange(k) + 0.5) * (L / k)
    src = np.stack(np.meshgrid(g, g, g, indexing="ij"), -1).reshape(-1, 3)
    acc = port.ewald(src, 1.0, 1.0, L, 0.1, src[::37], 8)
    newton_scale = 1.0 / (L / k) ** 2
    assert np.abs(acc).max() < 1e-10 * newton_scale


@pytest.mark.parametrize("dist", [0.003, 0.01, 0.03])
def test_close_pair_is_newton_plus_background(port, dist):
    L = 1.0
    d = np.array([0.6, -0.48, 0.64]) * dist  # |d| = dist
    src = np.array([[0.3, 0.4, 0.5]])
    tg = src - d  # d points from the target to the source
    acc = port.ewald(src, 1.0, 1.0, L, 1e-6, tg, 1)[0]
    expect = d / dist ** 3 - (4 * np.pi / 3) * d / L ** 3
    # the remainder is the cubic lattice's third-order term, ~5 (d/L)^5 relative
    assert np.abs(acc - expect).max() < 10 * dist ** 5 * np.linalg.norm(expect)


def test_softened_pair_uses_the_reference_spline(port):
    L, h = 1.0, 0.02
    src = np.array([[0.5, 0.5, 0.5]])
    out = []
    for u in (0.3, 0.7):  # both branches of the spline
        d = np.array([u * h, 0.0, 0.0])
        acc = port.ewald(src, 1.0, 1.0, L, h, src - d, 1)[0]
        if u < 0.5:
            fs = (10.66667 + u * u * (32.0 * u - 38.4)) / h ** 3
        else:
            fs = (21.33333 - 48.0 * u + 38.4 * u * u - 10.66667 * u ** 3 - 0.06667 / u ** 3) / h ** 3
        expect = fs * d - (4 * np.pi / 3) * d / L ** 3
        out.append(np.abs(acc - expect).max() / np.linalg.norm(expect))
    assert max(out) < 1e-7  # the O((d/L)^5) lattice remainder, as for the close pair


def test_error_metric():
    """rms relative error over all components, and the median and 99th
    percentile of the per-particle relative error (zero reference forces left
    out)."""
    from conftest import err_stats
    ref = np.array([[3.0, 0, 0], [0, 4.0, 0], [0, 0, 0], [1.0, 0, 0]])
    a = ref + np.array([[0.3, 0, 0], [0, 0, 0.4], [0.5, 0, 0], [0, 0.2, 0]])
    s = err_stats(a, ref)
    assert s["rms"] == pytest.approx(np.sqrt((0.09 + 0.16 + 0.25 + 0.04) / 26.0))
    assert s["median"] == pytest.approx(0.1)  # per particle: 0.1, 0.1, 0.2
    assert s["p99"] == pytest.approx(np.percentile([0.1, 0.1, 0.2], 99))
