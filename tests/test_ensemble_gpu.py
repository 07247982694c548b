"""Batched droplet ensembles: every box of a batch evolves as the same
configuration run alone (the same tile code and per-box constants, compiled
into different kernels, so within a few ulp), whatever the tuning; the
autotuner leaves the results unchanged."""
import numpy as np
import pytest

from conftest import rel_l2

pytestmark = pytest.mark.gpu

FIELDS = ("rho", "ux", "uy", "uz", "phi")


def small_batch(pf, n=5, vs=19):
    cfgs = pf.ensemble_configs(n=n, seed=7, velocity_set=vs)
    # keep the test quick: shrink the largest boxes
    for c in cfgs:
        e = min(int(c.nx), 48)
        c.nx = c.ny = c.nz = e
        c.radius = max(2, min(c.radius, e // 4))
        c.diam = 2 * c.radius
    return cfgs


@pytest.mark.parametrize("vs", [19, 27])
def test_boxes_match_single_runs(pflbm, vs):
    cfgs = small_batch(pflbm, vs=vs)
    steps = 37
    with pflbm.Ensemble(cfgs) as ens:
        ens.set_tuning(8, 2)
        ens.step(steps)
        got = [{f: ens.get_field(k, f) for f in FIELDS} for k in range(len(cfgs))]
    for k, c in enumerate(cfgs):
        with pflbm.Simulation(c) as s:
            s.step(steps)
            for f in FIELDS:
                tol = 1e-6 if f in ("rho", "phi") else 1e-3  # u: spurious currents ~1e-6
                assert rel_l2(got[k][f], s.get_field(f)) <= tol, (k, f)


def test_tuning_does_not_change_results(pflbm):
    cfgs = small_batch(pflbm, n=4)
    res = []
    for zc, ctas in ((4, 1), (64, 2)):
        with pflbm.Ensemble(cfgs) as ens:
            ens.set_tuning(zc, ctas)
            ens.step(20)
            res.append([ens.get_field(k, "phi") for k in range(len(cfgs))])
    for a, b in zip(*res):
        assert np.array_equal(a, b)


def test_autotune_and_mass(pflbm):
    cfgs = small_batch(pflbm, n=6)
    with pflbm.Ensemble(cfgs) as ens:
        best = ens.autotune(trial_steps=4)
        assert best["zchunk"] in (4, 8, 16, 32, 64) and best["ctas_per_sm"] in (1, 2, 3, 4)
        assert best["tile"] in ((32, 8), (32, 4), (64, 4), (32, 16))
        assert ens.tuning == {"tile": best["tile"], "zchunk": best["zchunk"], "ctas_per_sm": best["ctas_per_sm"]}
        ens.step(1)
        m0 = [ens.reduce(k).phi_mass for k in range(len(cfgs))]
        ens.step(100)
        for k in range(len(cfgs)):
            d = ens.reduce(k)
            assert d.nonfinite == 0
            assert abs(d.phi_mass - m0[k]) / m0[k] < 1e-6


@pytest.mark.parametrize("vs", [19, 27])
def test_tma_and_plain_batch_kernels_bit_identical(pflbm, monkeypatch, vs):
    """The TMA-fed batch collide (per-box tensor maps, pipeline barriers
    carried from tile to tile) and the float4 batch phase step compute
    exactly what the plain-load collide and the scalar phase step compute."""
    cfgs = small_batch(pflbm, n=5, vs=vs)
    out = {}
    for mode in ("tma", "plain"):
        if mode == "plain":
            monkeypatch.setenv("PFLBM_NO_TMA", "1")
            monkeypatch.setenv("PFLBM_NO_VEC", "1")
        with pflbm.Ensemble(cfgs) as ens:
            ens.set_tuning(8, 2)
            ens.step(23)
            out[mode] = [{f: ens.get_field(k, f) for f in FIELDS} for k in range(len(cfgs))]
    for k in range(len(cfgs)):
        for f in FIELDS:
            assert np.array_equal(out["tma"][k][f], out["plain"][k][f]), (k, f)


def test_unaligned_boxes_use_the_plain_path(pflbm):
    """Boxes whose rows are not 16-byte aligned (nx = 30, 34) run the
    plain-load collide and the scalar phase step; they still match single
    runs."""
    cfgs = small_batch(pflbm, n=3)
    for c, e in zip(cfgs, (30, 34, 32)):
        c.nx = c.ny = c.nz = e
        c.radius = e // 4
        c.diam = 2 * c.radius
    steps = 21
    with pflbm.Ensemble(cfgs) as ens:
        ens.step(steps)
        got = [{f: ens.get_field(k, f) for f in FIELDS} for k in range(len(cfgs))]
    for k, c in enumerate(cfgs):
        with pflbm.Simulation(c) as s:
            s.step(steps)
            for f in FIELDS:
                tol = 1e-6 if f in ("rho", "phi") else 1e-3
                assert rel_l2(got[k][f], s.get_field(f)) <= tol, (k, f)


@pytest.mark.parametrize("vs", [19, 27])
def test_tile_shapes_bit_identical(pflbm, vs):
    """The fused step's tile shapes (32x8, 32x4, 64x4, 32x16) change only how
    the grid is cut into work items: every node evaluates the same stencils
    and collision, so the fields are bit-identical whatever the shape."""
    cfgs = small_batch(pflbm, n=4, vs=vs)
    out = {}
    for tile in ((32, 8), (32, 4), (64, 4), (32, 16)):
        with pflbm.Ensemble(cfgs) as ens:
            ens.set_tile(*tile)
            assert ens.tuning["tile"] == tile
            ens.step(19)
            out[tile] = [ens.get_field(k, "phi") for k in range(len(cfgs))] + [
                ens.get_field(k, "uz") for k in range(len(cfgs))]
    ref = out[(32, 8)]
    for tile, v in out.items():
        for a, b in zip(v, ref):
            assert np.array_equal(a, b), tile
