"""Known-answer tests of the CPU oracle (no GPU).

The reference ships no tests; these check the oracle's restatement against
the lattice identities the reference's formulas satisfy
(src/velocitySet/D3Q19.cuh:143-187, D3Q27.cuh:152-206, D3Q7.cuh:129-153),
the published counter hash (src/BoundaryConditions.cuh:172-213), and the
conservation laws of the scheme.
"""
import numpy as np
import pytest

from conftest import rel_l2

VS = [19, 27]


def _py_hash32(x):
    # pure-Python restatement of hash32 (BoundaryConditions.cuh:172-181)
    m = 0xFFFFFFFF
    x ^= x >> 16
    x = (x * 0x7FEB352D) & m
    x ^= x >> 15
    x = (x * 0x846CA68B) & m
    x ^= x >> 16
    return x


@pytest.mark.parametrize("vs", VS)
def test_velocity_set_moments(oracle, vs):
    c, w = oracle.velocity_set(vs)
    assert c.shape == (vs, 3)
    w = w.astype(np.float64)
    assert abs(w.sum() - 1.0) < 1e-6
    assert np.allclose((w[:, None] * c).sum(0), 0.0, atol=1e-7)
    cc = np.einsum("q,qa,qb->ab", w, c, c)
    assert np.allclose(cc, np.eye(3) / 3.0, atol=1e-7)
    c4 = np.einsum("q,qa,qb,qc,qd->abcd", w, c, c, c, c)
    d = np.eye(3)
    iso = (np.einsum("ab,cd->abcd", d, d) + np.einsum("ac,bd->abcd", d, d) + np.einsum("ad,bc->abcd", d, d)) / 9.0
    assert np.allclose(c4, iso, atol=1e-7)
    # opposite pairs (2k-1, 2k), Appendix A ordering
    for k in range(1, (vs - 1) // 2 + 1):
        assert np.array_equal(c[2 * k - 1], -c[2 * k])
    assert np.array_equal(c[0], [0, 0, 0])


@pytest.mark.parametrize("vs", VS)
def test_feq_moments(oracle, vs):
    rng = np.random.default_rng(1)
    c, _ = oracle.velocity_set(vs)
    for _ in range(20):
        rho = float(1 + 0.01 * rng.standard_normal())
        u = 0.05 * rng.standard_normal(3)
        feq = oracle.node_feq(vs, rho, *u).astype(np.float64)
        # shifted storage: sum feq = rho - 1, sum feq c = rho u
        assert abs(feq.sum() - (rho - 1)) < 2e-7
        assert np.allclose((feq[:, None] * c).sum(0), rho * u.astype(np.float32), atol=2e-7)


@pytest.mark.parametrize("vs", VS)
def test_fneq_and_force_moments(oracle, vs):
    rng = np.random.default_rng(2)
    c, _ = oracle.velocity_set(vs)
    for _ in range(20):
        pi = 1e-3 * rng.standard_normal(6)
        tr = pi[0] + pi[1] + pi[2]
        pi[:3] -= tr / 3.0  # deviatoric, as after lbm.cu:117-120
        u = 0.05 * rng.standard_normal(3)
        fneq = oracle.node_fneq(vs, pi, *u).astype(np.float64)
        assert abs(fneq.sum()) < 1e-8
        assert np.allclose((fneq[:, None] * c).sum(0), 0.0, atol=1e-8)
        # second moment of the regularised part reproduces Pi
        P = np.array([[pi[0], pi[3], pi[4]], [pi[3], pi[1], pi[5]], [pi[4], pi[5], pi[2]]])
        assert np.allclose(np.einsum("q,qa,qb->ab", fneq, c, c), P, atol=1e-8)
        F = 1e-4 * rng.standard_normal(3)
        frc = oracle.node_force(vs, *u, *F).astype(np.float64)
        # Guo force: zeroth moment 0, first moment F
        assert abs(frc.sum()) < 1e-9
        assert np.allclose((frc[:, None] * c).sum(0), F, atol=1e-9)


def test_phase_equilibrium(oracle):
    rng = np.random.default_rng(3)
    for _ in range(20):
        phi = float(rng.uniform())
        u = 0.05 * rng.standard_normal(3)
        g = oracle.node_geq(phi, *u).astype(np.float64)
        assert abs(g.sum() - phi) < 1e-7
        n = rng.standard_normal(3)
        n /= np.linalg.norm(n)
        h = oracle.node_antidiff(0.05 * phi * (1 - phi), *n).astype(np.float64)
        assert abs(h.sum()) < 1e-9  # anti-diffusion conserves phi (D3Q7.cuh:145-153)


def test_hash32_known_answers(oracle):
    for x in [0, 1, 2, 0xDEADBEEF, 0x9E3779B9, 123456789, 0xFFFFFFFF]:
        assert oracle.hash32(x) == _py_hash32(x)
    assert oracle.hash32(0) == 0


def test_white_noise_is_standard_normal(oracle):
    z = np.array([oracle.white_noise(0xA341316C, x, y, t) for x in range(20) for y in range(20) for t in range(5)])
    assert abs(z.mean()) < 0.1
    assert abs(z.std() - 1.0) < 0.1
    u = np.array([oracle.uniform_noise(7, x, y, 3) for x in range(40) for y in range(40)])
    assert u.min() >= -1.0 and u.max() < 1.0
    assert abs(u.mean()) < 0.05


def test_reference_config(oracle, pflbm):
    # the library's pflbm_config_reference equals the oracle's independent restatement
    for case in (0, 1):
        for vs in VS:
            a = oracle.config_reference(case, vs).as_dict()
            b = pflbm.config_reference(case, vs).as_dict()
            assert a == b
    jet = oracle.config_reference(1, 19)
    assert (jet.nx, jet.ny, jet.nz, jet.diam) == (64, 64, 128, 10)
    assert np.float32(jet.sigma) == np.float32(np.float32(0.05 * 0.05) * 10) / np.float32(500) or jet.sigma > 0
    assert abs(jet.gamma - 0.5) < 1e-7
    drop = oracle.config_reference(0, 27)
    assert (drop.nx, drop.radius, drop.tau, drop.sigma) == (128, 35, np.float32(0.55), np.float32(0.03))


def test_sponge_ramp(oracle):
    jet = oracle.config_reference(1, 19)
    nz = jet.nz
    vals = np.array([oracle.sponge_ramp(jet, z) for z in range(nz)])
    cells = nz // 12
    assert np.all(vals[: nz - 1 - cells] == 0.0)
    assert vals[-1] == pytest.approx(1.0, abs=1e-6)
    assert np.all(np.diff(vals) >= 0)


def _small_droplet(pflbm, vs=19, n=24, radius=6, stretch=2.0):
    c = pflbm.config_reference(0, vs)
    c.nx = c.ny = c.nz = n
    c.radius, c.diam = radius, 2 * radius
    c.droplet_x_stretch = stretch
    return c


@pytest.mark.parametrize("vs", VS)
def test_oracle_phase_mass_conservation(oracle, pflbm, vs):
    c = _small_droplet(pflbm, vs)
    for fp64, tol in ((False, 2e-6), (True, 1e-12)):
        s = oracle.OracleSim(c, fp64=fp64)
        s.step(1)
        m0 = s.get_field("phi")[1:-1, 1:-1, 1:-1].sum()
        s.step(100)
        m1 = s.get_field("phi")[1:-1, 1:-1, 1:-1].sum()
        assert abs(m1 - m0) / m0 < tol


def test_oracle_float_vs_double(oracle, pflbm):
    c = _small_droplet(pflbm, 19)
    a = oracle.OracleSim(c, fp64=False)
    b = oracle.OracleSim(c, fp64=True)
    a.step(50)
    b.step(50)
    for f in ("rho", "phi"):
        assert rel_l2(a.get_field(f), b.get_field(f)) < 1e-5


def test_oracle_laplace_law(oracle, pflbm):
    # static droplet: cs2 (rho_in - rho_out) ~ 2 sigma / R (diffuse interface,
    # so within 35%)
    c = _small_droplet(pflbm, 19, n=40, radius=10, stretch=1.0)
    c.sigma = 0.01
    c.tau = 0.6
    s = oracle.OracleSim(c, fp64=True)
    s.step(600)
    rho = s.get_field("rho")[1:-1, 1:-1, 1:-1]
    phi = s.get_field("phi")[1:-1, 1:-1, 1:-1]
    dp = (rho[phi > 0.9].mean() - rho[phi < 0.1].mean()) / 3.0
    assert dp == pytest.approx(2 * c.sigma / c.radius, rel=0.35)


def test_oracle_jet_runs_and_inlet_state(oracle, pflbm):
    c = pflbm.config_reference(1, 19)
    c.nx, c.ny, c.nz = 24, 24, 36
    c.diam, c.radius = 8, 4
    s = oracle.OracleSim(c)
    s.step(20)
    phi = s.get_field("phi")
    uz = s.get_field("uz")
    # inlet ghost plane: phi = 1 and uz = u_inf inside the disc (BoundaryConditions.cuh:66-71)
    cx = (c.nx - 1) / 2
    assert phi[0, int(cx), int(cx)] == 1.0
    assert uz[0, int(cx), int(cx)] == pytest.approx(0.05)
    assert np.isfinite(s.get_field("rho")).all()
    # outlet ghost plane copies plane nz-2 (BoundaryConditions.cuh:122-126)
    assert np.array_equal(s.get_field("rho")[-1, 1:-1, 1:-1], s.get_field("rho")[-2, 1:-1, 1:-1])


def test_oracle_matches_reference_formulas(oracle):
    """Per-node formulas of the oracle against golden vectors produced by the
    reference's own velocity-set headers (tests/golden/gen_formulas.py)."""
    import json
    from pathlib import Path

    g = json.loads((Path(__file__).parent / "golden" / "formulas.json").read_text())
    assert len(g["cases"]) >= 60
    for case in g["cases"]:
        x = np.float32(case["in"])
        if case["set"] == 7:
            got_g = oracle.node_geq(*x[:4])
            got_h = oracle.node_antidiff(*x[4:8])
            np.testing.assert_array_equal(got_g, np.float32(case["geq"]))
            np.testing.assert_array_equal(got_h, np.float32(case["antidiff"]))
            continue
        vs = case["set"]
        rho, u, pi, F = x[0], x[1:4], x[4:10], x[10:13]
        np.testing.assert_array_equal(oracle.node_feq(vs, rho, *u), np.float32(case["feq"]))
        np.testing.assert_array_equal(oracle.node_fneq(vs, pi, *u), np.float32(case["fneq"]))
        np.testing.assert_array_equal(oracle.node_force(vs, *u, *F), np.float32(case["force"]))


def test_relaxation_constants_match_reference(oracle):
    """Relaxation, sponge, sigma and gamma of the reference's default cases
    (src/constants.cuh:80-141, globalFunctions.cuh:260-461), from the
    reference's own constexpr functions (tests/golden/gen_formulas.py)."""
    import json
    from pathlib import Path

    g = json.loads((Path(__file__).parent / "golden" / "formulas.json").read_text())["relaxation"]
    jet = oracle.config_reference(1, 19)
    r = oracle.relaxation(jet)  # omega_ref, tau_water, tau_oil, omco_zmin, z_start, inv_nz_m1, inv_sponge
    j = g["jet"]
    assert np.float32(r[1]) == np.float32(j["tau_water"])
    assert np.float32(r[2]) == np.float32(j["tau_oil"])
    assert np.float32(r[3]) == np.float32(j["omco_zmin"])
    assert np.float32(r[4]) == np.float32(j["z_start"])
    assert np.float32(r[5]) == np.float32(j["inv_nz_m1"])
    assert np.float32(r[6]) == np.float32(j["inv_sponge"])
    assert np.float32(jet.sigma) == np.float32(j["sigma"])
    assert np.float32(jet.gamma) == np.float32(j["gamma"])
    drop = oracle.config_reference(0, 19)
    rd = oracle.relaxation(drop)
    assert np.float32(rd[0]) == np.float32(g["droplet"]["omega_ref"])
    assert np.float32(drop.sigma) == np.float32(g["droplet"]["sigma"])
