"""The interface-width estimator of the closure's phase-field part
(pflbm_closure_interface_scale), W = 4 sum phi(1-phi) / sum |grad phi| with
the solver's D3Q19 lattice gradient, on known profiles (numpy only): it
recovers the width of tanh interfaces, and a profile resolved on a 2x finer
grid gives twice the width in its own lattice units, the ratio the closure
turns into its sharpening scale."""
import itertools

import numpy as np
import pytest

# D3Q19: rest, 6 axis (w 1/18), 12 face diagonals (w 1/36)
C = np.array([c for c in itertools.product((-1, 0, 1), repeat=3) if sum(abs(v) for v in c) <= 2])
W = np.array([1 / 3 if not c.any() else (1 / 18 if abs(c).sum() == 1 else 1 / 36) for c in C])


def lattice_grad_norm(phi):
    """3 |sum_q w_q c_q phi(x + c_q)| on a periodic grid (arrays are z, y, x)."""
    g = np.zeros((3,) + phi.shape)
    for c, w in zip(C, W):
        sh = np.roll(phi, shift=(-c[2], -c[1], -c[0]), axis=(0, 1, 2))
        for a in range(3):
            g[a] += w * c[a] * sh
    return 3.0 * np.sqrt((g ** 2).sum(axis=0))


def width(phi, interior):
    ind = lattice_grad_norm(phi)
    return 4.0 * np.sum((phi * (1 - phi))[interior]) / np.sum(ind[interior])


@pytest.mark.parametrize("w", [4.0, 8.0, 16.0])
def test_planar_tanh_width(w):
    nx = 256
    x = np.arange(nx, dtype=np.float64)
    # a slab between two interfaces, periodic in x so that the roll is exact
    prof = 0.5 * (np.tanh(2 * (x - nx / 4) / w) - np.tanh(2 * (x - 3 * nx / 4) / w))
    phi = np.broadcast_to(prof, (4, 4, nx)).copy()
    got = width(phi, np.ones_like(phi, dtype=bool))
    assert got == pytest.approx(w, rel=0.02)


def test_spherical_droplet_width():
    n, r, w = 96, 24.0, 6.0
    z, y, x = np.meshgrid(*(np.arange(n, dtype=np.float64),) * 3, indexing="ij")
    d = np.sqrt((x - n / 2) ** 2 + (y - n / 2) ** 2 + (z - n / 2) ** 2)
    phi = 0.5 + 0.5 * np.tanh(2 * (r - d) / w)
    assert width(phi, np.ones_like(phi, dtype=bool)) == pytest.approx(w, rel=0.03)


def test_finer_grid_doubles_the_width_in_lattice_units():
    # one physical profile (width 5 coarse cells) sampled on a coarse grid and
    # on a grid twice as fine: the width in each grid's own units differs by 2
    w_phys, nxc = 5.0, 128
    xc = np.arange(nxc, dtype=np.float64)
    xf = np.arange(2 * nxc, dtype=np.float64) / 2.0
    prof = lambda x: 0.5 * (np.tanh(2 * (x - nxc / 4) / w_phys) - np.tanh(2 * (x - 3 * nxc / 4) / w_phys))
    coarse = np.broadcast_to(prof(xc), (4, 4, nxc)).copy()
    fine = np.broadcast_to(prof(xf), (4, 4, 2 * nxc)).copy()
    wc = width(coarse, np.ones_like(coarse, dtype=bool))
    wf = width(fine, np.ones_like(fine, dtype=bool))
    assert wf / wc == pytest.approx(2.0, rel=0.03)
