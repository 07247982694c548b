"""Parity of the CUDA library (through the C ABI) with the CPU oracle.

The oracle restates the reference's passes (src/phaseField.cuh, src/lbm.cu,
src/BoundaryConditions.cuh) with its single-buffer push; the library runs the
fused two-kernel pull step. Tolerances:
  * FP64 storage vs FP64 oracle: rel. L2 <= 1e-10 on every field. Only
    summation order differs, so this pins the semantics (ghost shell, BCs,
    step order, noise) exactly. The reference's Gaussian inflow noise is
    computed in float with logf/cosf, whose last-ulp results differ between
    the host libm and CUDA; jets in that mode are held to 1e-7 instead.
  * FP32 vs FP32 oracle: rel. L2 <= 1e-5 on rho and phi. The velocity of a
    static droplet or a young jet is small, and its relative L2 floor in any
    FP32 implementation, measured here as the oracle's own FP32-vs-FP64
    difference on the same case and horizon, lies between 3e-6 and 5e-5; u
    (the vector field and each component) must be within
    max(1e-5, 2 x floor). Pi and F, small differences of large terms, are
    held to 1e-3.
"""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

BASIC = ("rho", "ux", "uy", "uz", "phi")
AVG_FIELDS = ("avg_phi", "avg_ux", "avg_uy", "avg_uz", "avg_uxux", "avg_uyuy", "avg_uzuz", "avg_uxuy",
              "avg_uxuz", "avg_uyuz")
ALL18 = ("rho", "ux", "uy", "uz", "pxx", "pyy", "pzz", "pxy", "pxz", "pyz",
         "phi", "normx", "normy", "normz", "ind", "fsx", "fsy", "fsz")


def droplet_cfg(pf, vs, n=32, radius=8, stretch=2.0, **kw):
    c = pf.config_reference(pf.CASE_DROPLET, vs)
    c.nx = c.ny = c.nz = n
    c.radius, c.diam = radius, 2 * radius
    c.droplet_x_stretch = stretch
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def jet_cfg(pf, vs, nx=32, ny=32, nz=64, diam=10, noise=0, **kw):
    c = pf.config_reference(pf.CASE_JET, vs)
    c.nx, c.ny, c.nz = nx, ny, nz
    c.diam, c.radius = diam, diam // 2
    c.inflow_noise = noise
    if noise == 1:
        c.noise_amp = 0.05
        c.seed = 99
    for k, v in kw.items():
        setattr(c, k, v)
    return c


def run_pair(pf, oracle, cfg, steps, fp64=False, fields=BASIC, floor=False):
    c = cfg.copy()
    c.storage = pf.STORAGE_FP64 if fp64 else pf.STORAGE_FP32
    o = oracle.OracleSim(c, fp64=fp64)
    o.step(steps)
    with pf.Simulation(c) as s:
        s.step(steps)
        assert s.current_step == steps
        lib = {f: s.get_field(f, dtype=np.float64) for f in fields}
    ora = {f: o.get_field(f) for f in fields}
    errs = {f: rel_l2(lib[f], ora[f]) for f in fields}
    if "ux" in fields:
        errs["u"] = rel_l2(np.stack([lib[f] for f in ("ux", "uy", "uz")]), np.stack([ora[f] for f in ("ux", "uy", "uz")]))
    if floor:
        o64 = oracle.OracleSim(c, fp64=True)
        o64.step(steps)
        fl = {f: rel_l2(ora[f], o64.get_field(f)) for f in ("rho", "ux", "uy", "uz", "phi")}
        fl["u"] = rel_l2(np.stack([ora[f] for f in ("ux", "uy", "uz")]),
                         np.stack([o64.get_field(f) for f in ("ux", "uy", "uz")]))
        errs["floor"] = fl
    return errs


CASES = [
    ("droplet19", lambda pf: droplet_cfg(pf, 19), 120),
    ("droplet27", lambda pf: droplet_cfg(pf, 27), 120),
    ("jet19", lambda pf: jet_cfg(pf, 19), 80),
    ("jet27", lambda pf: jet_cfg(pf, 27), 80),
    ("jet19_uniform", lambda pf: jet_cfg(pf, 19, noise=1), 80),
    ("jet27_uniform_odd", lambda pf: jet_cfg(pf, 27, nx=30, ny=34, nz=40, diam=8, noise=1), 37),
]


@pytest.mark.parametrize("name,make,steps", CASES, ids=[c[0] for c in CASES])
def test_fp64_semantics(pflbm, oracle, name, make, steps):
    cfg = make(pflbm)
    tol = 1e-7 if (cfg.flow_case == pflbm.CASE_JET and cfg.inflow_noise == pflbm.NOISE_GAUSSIAN_UXY) else 1e-10
    errs = run_pair(pflbm, oracle, cfg, steps, fp64=True, fields=ALL18)
    bad = {k: v for k, v in errs.items() if not v <= tol}
    assert not bad, bad


@pytest.mark.parametrize("name,make,steps", CASES, ids=[c[0] for c in CASES])
def test_fp32_parity(pflbm, oracle, name, make, steps):
    errs = run_pair(pflbm, oracle, make(pflbm), steps, fp64=False, fields=ALL18, floor=True)
    floor = errs.pop("floor")
    bad = {k: errs[k] for k in ("rho", "phi") if not errs[k] <= 1e-5}
    bad.update({k: errs[k] for k in ("u", "ux", "uy", "uz") if not errs[k] <= max(1e-5, 2.0 * floor[k])})
    bad.update({k: v for k, v in errs.items() if k not in BASIC + ("u",) and not v <= 1e-3})
    assert not bad, (errs, floor)


@pytest.mark.parametrize("steps", [0, 1, 2, 3, 17])
def test_step_counts_and_initial_state(pflbm, oracle, steps):
    # odd/even counts exercise every captured graph (1, 2, 16 steps)
    errs = run_pair(pflbm, oracle, jet_cfg(pflbm, 19, nx=24, ny=24, nz=30, diam=6, noise=1), steps, fp64=True)
    assert max(errs.values()) <= 1e-10, errs


def test_split_stepping_equals_one_call(pflbm):
    c = jet_cfg(pflbm, 27, nx=24, ny=24, nz=40, diam=8)
    with pflbm.Simulation(c) as a, pflbm.Simulation(c) as b:
        a.step(40)
        for k in (1, 2, 16, 5, 16):
            b.step(k)
        for f in BASIC:
            assert np.array_equal(a.get_field(f), b.get_field(f))


def test_reinit_is_deterministic(pflbm):
    c = droplet_cfg(pflbm, 19, n=24, radius=6)
    with pflbm.Simulation(c) as s:
        s.step(30)
        r1 = s.get_field("phi").copy()
        s.init()
        s.step(30)
        assert np.array_equal(r1, s.get_field("phi"))


def test_phase_mass_conservation_droplet64(pflbm):
    # the plain static droplet preset (gamma = 0.05): phi mass conserved to
    # 1e-6 relative over 1000 steps
    c = pflbm.preset("droplet64")
    with pflbm.Simulation(c) as s:
        s.step(1)
        m0 = s.reduce().phi_mass
        s.step(999)
        d = s.reduce()
        assert d.nonfinite == 0
        assert abs(d.phi_mass - m0) / m0 < 1e-6


def test_laplace_law_droplet64(pflbm):
    # With tau_g = 1 the phase diffusivity is M = cs2/2 = 1/8, and the interface
    # keeps the width W = 4 only for gamma = 4 M / (W cs2) = 0.5
    # (src/constants.cuh:104-108); gamma = 0.05 relaxes to a 40-cell
    # interface. The Laplace jump is therefore checked with gamma = 0.5:
    # cs2 (rho_in - rho_out) within 35% of 2 sigma / R (diffuse interface).
    c = pflbm.preset("droplet64", gamma=0.5)
    with pflbm.Simulation(c) as s:
        s.step(1000)
        d = s.reduce()
        assert d.n_in > 1000 and d.n_out > 1000
        assert d.laplace_dp == pytest.approx(2 * c.sigma / c.radius, rel=0.35)


def test_derived_fields_match_oracle(pflbm, oracle):
    c = jet_cfg(pflbm, 19, nx=24, ny=24, nz=36, diam=8, noise=1)
    c.flags = pflbm.FLAG_TIME_AVERAGE | pflbm.FLAG_REYNOLDS_MOMENTS | pflbm.FLAG_VORTICITY
    c.storage = pflbm.STORAGE_FP64
    o = oracle.OracleSim(c, fp64=True)
    o.step(25)
    with pflbm.Simulation(c) as s:
        s.step(25)
        for f in ("avg_phi", "avg_ux", "avg_uy", "avg_uz", "avg_uxux", "avg_uyuy", "avg_uzuz",
                  "avg_uxuy", "avg_uxuz", "avg_uyuz", "vort_x", "vort_y", "vort_z", "vort_mag"):
            assert rel_l2(s.get_field(f, dtype=np.float64), o.get_field(f)) <= 1e-10, f


# 16-bit storage against FP32 storage on the same young jet (60 steps,
# reference physics): rel. L2 bounds about 2-5x the measured FP16 (rho
# 3.9e-7, u 3.8e-4, phi 7.3e-6) and BF16 (rho 4.4e-6, u 4.4e-3, phi 1.2e-4)
# differences
LOW_PRECISION_TOL = {
    1: {"rho": 2e-6, "ux": 1e-3, "uy": 1e-3, "uz": 5e-4, "phi": 3e-5},
    2: {"rho": 2e-5, "ux": 1e-2, "uy": 1e-2, "uz": 5e-3, "phi": 5e-4},
}


def test_low_precision_storage_close_to_fp32(pflbm):
    c = jet_cfg(pflbm, 19, nx=32, ny=32, nz=48, diam=8)
    with pflbm.Simulation(c) as s:
        s.step(60)
        ref = {f: s.get_field(f) for f in BASIC}
    for st in (pflbm.STORAGE_FP16, pflbm.STORAGE_BF16):
        c2 = c.copy()
        c2.storage = st
        with pflbm.Simulation(c2) as s:
            s.step(60)
            e = {f: rel_l2(s.get_field(f), ref[f]) for f in BASIC}
        print("storage", st, e)
        bad = {f: v for f, v in e.items() if not v <= LOW_PRECISION_TOL[st][f]}
        assert not bad, (st, bad, e)


def test_write_output_layout(pflbm, tmp_path):
    c = droplet_cfg(pflbm, 19, n=16, radius=4)
    with pflbm.Simulation(c) as s:
        s.step(3)
        s.write_output(tmp_path, ("rho", "uz", "phi"))
        n = c.nodes
        for name in ("rho", "uz", "phi"):
            b = tmp_path / f"{name}000002.bin"
            assert b.stat().st_size == 4 * n
            assert np.array_equal(np.fromfile(b, np.float32).reshape(16, 16, 16), s.get_field(name))
        vti = (tmp_path / "step_000002.vti").read_bytes()
        assert vti.startswith(b'<?xml version="1.0"?>')
        assert b'WholeExtent="0 15 0 15 0 15"' in vti
        assert b'Name="uz" NumberOfComponents="1" format="appended" offset="16388"' in vti


@pytest.mark.parametrize("vs,storage,avg", [(19, 0, 0), (27, 0, 0), (19, 1, 0), (27, 2, 0), (19, 3, 0), (27, 0, 1)])
def test_tma_and_vector_paths_bit_identical(pflbm, monkeypatch, vs, storage, avg):
    # The TMA-fed collide kernel and the float4 phase kernel compute exactly
    # what the plain-load kernels compute; only the data movement differs
    # (avg: the collide mode that also updates the time averages).
    # (one node per thread: the node-pair kernel is compared below)
    c = jet_cfg(pflbm, vs, nx=64, ny=40, nz=48, diam=10, noise=1)
    c.storage = storage
    if avg:
        c.flags = pflbm.FLAG_TIME_AVERAGE | pflbm.FLAG_REYNOLDS_MOMENTS
    fields = ALL18 + (AVG_FIELDS if avg else ())
    out = {}
    monkeypatch.setenv("PFLBM_NO_PAIR", "1")
    for mode in ("fast", "plain"):
        if mode == "plain":
            monkeypatch.setenv("PFLBM_NO_TMA", "1")
            monkeypatch.setenv("PFLBM_NO_VEC", "1")
        with pflbm.Simulation(c) as s:
            if mode == "fast":
                assert s.uses_tma and s.collide_variant == "tma"
            else:
                assert not s.uses_tma and s.collide_variant == "plain"
            s.step(33)
            out[mode] = {f: s.get_field(f, dtype=np.float64) for f in fields}
    for f in fields:
        assert np.array_equal(out["fast"][f], out["plain"][f]), f


PAIR_TOL = {  # rel. L2 of the node-pair kernel against the one-node kernel: rho, phi, u
    0: (1e-6, 1e-6, 3e-5),    # FP32: rounding of the reordered algebra
    1: (1e-5, 5e-5, 2e-3),    # FP16: the last stored bit differs now and then
    2: (5e-5, 5e-4, 1e-2),    # BF16
}
# FP32 droplets: the velocity is spurious currents, whose FP32 rounding floor
# (the oracle's own FP32-vs-FP64 difference) reaches 5e-5; the reordered
# algebra's rounding shows as u 2.8e-5 and phi 2.2e-6 after 60 steps of the
# R = 10 droplet
PAIR_TOL_FP32_DROPLET = (1e-6, 5e-6, 6e-5)


@pytest.mark.parametrize("case,vs,storage", [
    ("jet", 19, 1), ("droplet", 19, 1), ("jet", 19, 2), ("jet_overhang", 19, 1),
    ("jet", 19, 0), ("droplet", 19, 0), ("jet", 27, 0), ("droplet", 27, 0), ("jet", 27, 1),
])
def test_pair_kernel_matches_one_node_kernel(pflbm, monkeypatch, case, vs, storage):
    # The node-pair collide (two x-adjacent nodes per thread, packed FP32x2
    # arithmetic, default for 16-bit D3Q19) against the one-node TMA kernel.
    # FP32 and D3Q27 run it only when PFLBM_PAIR=1 selects it; the FP32
    # cases pin its algebra at FP32 rounding. jet_overhang: nx = 72, the
    # last column tile extends past the grid.
    if case == "droplet":
        c = droplet_cfg(pflbm, vs, n=48, radius=10)
        steps = 60
    elif case == "jet_overhang":
        c = jet_cfg(pflbm, vs, nx=72, ny=36, nz=40, diam=8, noise=1)
        steps = 25
    else:
        c = jet_cfg(pflbm, vs, nx=64, ny=40, nz=48, diam=10, noise=1)
        steps = 33
    c.storage = storage
    out = {}
    for mode in ("pair", "one"):
        if mode == "pair":
            monkeypatch.setenv("PFLBM_PAIR", "1")
        else:
            monkeypatch.delenv("PFLBM_PAIR", raising=False)
            monkeypatch.setenv("PFLBM_NO_PAIR", "1")
        with pflbm.Simulation(c) as s:
            assert s.collide_variant == ("tma_pairs" if mode == "pair" else "tma")
            s.step(steps)
            out[mode] = {f: s.get_field(f, dtype=np.float64) for f in BASIC}
    t_rho, t_phi, t_u = PAIR_TOL_FP32_DROPLET if (storage == 0 and case == "droplet") else PAIR_TOL[storage]
    e = {f: rel_l2(out["pair"][f], out["one"][f]) for f in BASIC}
    e["u"] = rel_l2(np.stack([out["pair"][f] for f in ("ux", "uy", "uz")]),
                    np.stack([out["one"][f] for f in ("ux", "uy", "uz")]))
    assert e["rho"] <= t_rho and e["phi"] <= t_phi and e["u"] <= t_u, e


def test_pair_kernel_is_the_default_for_16bit_d3q19(pflbm, monkeypatch):
    monkeypatch.delenv("PFLBM_PAIR", raising=False)
    monkeypatch.delenv("PFLBM_NO_PAIR", raising=False)
    for vs, storage, want in ((19, 1, "tma_pairs"), (19, 2, "tma_pairs"), (19, 0, "tma"), (27, 1, "tma"),
                              (27, 0, "tma"), (19, 3, "tma")):
        c = jet_cfg(pflbm, vs, nx=64, ny=40, nz=48, diam=10)
        c.storage = storage
        with pflbm.Simulation(c) as s:
            assert s.collide_variant == want, (vs, storage)


@pytest.mark.parametrize("storage", [0, 1])
def test_checkpoint_resume_bit_identical(pflbm, tmp_path, storage):
    c = jet_cfg(pflbm, 27, nx=32, ny=32, nz=48, diam=8, noise=1)
    c.storage = storage
    c.flags = pflbm.FLAG_TIME_AVERAGE
    ck = tmp_path / "state.ckpt"
    with pflbm.Simulation(c) as a:
        a.step(31)
        a.save_checkpoint(ck)
        a.step(20)
        want = {f: a.get_field(f) for f in BASIC + ("avg_uz",)}
    with pflbm.Simulation(c) as a2:
        a2.step(31)
        at31 = {f: a2.get_field(f) for f in ALL18}
    with pflbm.Simulation(c, init=False) as b:
        b.load_checkpoint(ck)
        assert b.current_step == 31
        for f in ALL18:  # readback right after a load is the step-31 state
            assert np.array_equal(b.get_field(f), at31[f]), f
        b.step(20)
        for f, v in want.items():
            assert np.array_equal(b.get_field(f), v), f
    bad = c.copy()
    bad.nz = 50
    with pflbm.Simulation(bad, init=False) as d:
        with pytest.raises(pflbm.PflbmError):
            d.load_checkpoint(ck)
