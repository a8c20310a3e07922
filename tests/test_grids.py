"""Domains of several voxel grids (ComputationalDomain::voxel_grids_, first-hit order,
src/MIDSX/Core/computational_domain.cpp:23-31): the oracle on CPU, and the GPU kernels
against the oracle on the same Philox streams (FP64: history by history) and statistically
(mixed form)."""
import numpy as np
import pytest

import midsx_gb300 as M
import oracle
from midsx_gb300 import native as N
from midsx_gb300 import scenes


def three_grid_scene():
    """Three grids in a 10.7 x 9.2 x 8.2 cm air domain, as in the reference's lead-attenuation
    example (cpp_simulations/lead_attenuation/lead_attenuation.json has three grids with their
    own origins), with synthetic voxel data: a lead block near the source (0.5 mm voxels), a
    detector slab of water and soft tissue (1 mm voxels), and a second lead block that overlaps
    the slab, where the slab - listed first - owns the overlap."""
    block = np.full((16, 20, 10), scenes.LEAD, dtype=np.uint8)        # 0.5 x 1.0 x 0.8 cm
    slab = np.full((40, 60, 4), scenes.WATER, dtype=np.uint8)         # 0.4 x 6.0 x 4.0 cm
    slab[10:30, 20:40, :] = scenes.SOFT_TISSUE
    grids = [(block, (0.05, 0.05, 0.05), (2.0, 5.0, 4.5)),
             (slab, (0.1, 0.1, 0.1), (9.65, 0.2, 1.6)),
             (block, (0.05, 0.05, 0.05), (9.8, 3.0, 3.0))]
    domain = (10.7, 9.2, 8.2)
    # the reference example's source: a point on the x = 0 face emitting towards the whole
    # far plane (RectangularIsotropicDirectionality)
    source = dict(position=(0.0, 4.6, 4.1), direction=("rect", (9.65, 0.0, 0.0), (0, 9.2, 0), (0, 0, 8.2)),
                  energy=60e3)
    return domain, grids, source


MATERIALS = [scenes.AIR, scenes.WATER, scenes.SOFT_TISSUE, scenes.LEAD]


def test_oracle_single_grid_list_equals_single_grid():
    sc = scenes.water_cube(n_histories=1, n=20, bins=4)
    blob = oracle.tables_for(sc)
    kw = sc.oracle_kwargs()
    a = oracle.run(blob, n=20_000, seed=3, threads=2, **kw)
    b = oracle.run(blob, n=20_000, seed=3, threads=2, grids=[(sc.ids, sc.spacing, sc.origin)], **kw)
    assert a["stats"] == b["stats"]
    for k in ("sum", "sumsq", "count"):
        np.testing.assert_array_equal(a["dose"][k], b["dose"][k][0])


def test_oracle_first_grid_wins():
    """A second grid lying wholly inside the first is never reached: the transport equals the
    first grid alone, and the second grid's dose stays zero."""
    sc = scenes.water_cube(n_histories=1, n=20, bins=4)
    blob = oracle.tables_for(sc)
    kw = sc.oracle_kwargs()
    inner = np.full((4, 4, 4), scenes.AIR, dtype=np.uint8)
    a = oracle.run(blob, n=20_000, seed=4, threads=2, **kw)
    b = oracle.run(blob, n=20_000, seed=4, threads=2, grids=[(sc.ids, sc.spacing, sc.origin),
                                                             (inner, (0.5, 0.5, 0.5), (8, 8, 8))], **kw)
    assert a["stats"] == b["stats"]
    np.testing.assert_array_equal(a["dose"]["sum"], b["dose"]["sum"][0])
    assert not b["dose"]["count"][1].any()


@pytest.mark.gpu
def test_grids_fp64_histories_equal_oracle():
    domain, grids, source = three_grid_scene()
    tables = M.Tables(MATERIALS, e_max=100e3)
    ph = M.Phantom.from_grids(tables, domain, scenes.AIR, grids)
    src = M.Source(**source)
    n = 60_000
    g = M.trace_deposits(tables, ph, src, n, seed=12, precision="fp64")
    o = oracle.run(oracle.tables_like(tables), domain, None, None, None, scenes.AIR, source, n=n, seed=12, history=True,
                   dose=False, grids=grids)["history_deposit"]
    same = np.abs(g - o) <= 1e-9 * np.maximum(1.0, np.abs(o))
    assert o.sum() > 0 and same.mean() > 0.999, same.mean()


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_grids_dose_against_oracle(precision):
    """Per-grid dose: totals and voxel z-scores against an independent oracle run."""
    domain, grids, source = three_grid_scene()
    tables = M.Tables(MATERIALS, e_max=100e3)
    ph = M.Phantom.from_grids(tables, domain, scenes.AIR, grids)
    src = M.Source(**source)
    tl = M.Tallies(ph, (), N.DOSE_FULL)
    n = 300_000
    M.run(tables, ph, src, tl, n, seed=5, precision=precision)
    d = tl.dose()
    st = tl.stats()
    o = oracle.run(oracle.tables_like(tables), domain, None, None, None, scenes.AIR, source, n=n, seed=6, rng=oracle.RNG_MT19937,
                   grids=grids)
    assert len(d["sum"]) == 3 and d["sum"][2].shape == grids[2][0].shape
    # all grids together: most of the deposit is whole-photon absorption in lead, so the
    # total's relative spread is ~0.5 % at this size; compare by z-score
    q = sum(d["sumsq"][k].sum() + o["dose"]["sumsq"][k].sum() for k in range(3))
    assert abs(st["deposited_grid"] - o["stats"]["deposited_grid"]) / np.sqrt(q) < 4
    for k in range(3):
        # the grid's total deposit: z-score with the deposit-based variance of both runs
        gs, os_ = d["sum"][k].sum(), o["dose"]["sum"][k].sum()
        zt = (gs - os_) / np.sqrt(d["sumsq"][k].sum() + o["dose"]["sumsq"][k].sum())
        assert os_ > 0 and abs(zt) < 4, (k, gs, os_, zt)
        s1, q1 = d["sum"][k].ravel(), d["sumsq"][k].ravel()
        s2, q2 = o["dose"]["sum"][k].ravel(), o["dose"]["sumsq"][k].ravel()
        sel = (s1 + s2) > 0.01 * max(s1.max(), s2.max())
        z = (s1[sel] - s2[sel]) / np.sqrt(q1[sel] + q2[sel])
        assert np.mean(np.abs(z) > 3) < 0.02, (k, np.mean(np.abs(z) > 3))


@pytest.mark.gpu
def test_one_grid_list_equals_single_grid_phantom():
    sc = scenes.water_cube(n_histories=1, n=30, bins=4)
    tables = M.Tables(sc.materials, e_max=sc.e_max)
    src = M.Source(**sc.source)
    a_ph = M.Phantom(tables, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
    b_ph = M.Phantom.from_grids(tables, sc.domain, sc.background, [(sc.ids, sc.spacing, sc.origin)])
    out = []
    for ph in (a_ph, b_ph):
        tl = M.Tallies(ph, sc.specs, N.DOSE_FULL)
        M.run(tables, ph, src, tl, 50_000, seed=2, precision="mixed")
        out.append((tl.dose()["sum"], tl.binned(0)[0], tl.stats()))
    np.testing.assert_array_equal(out[0][0], out[1][0])
    np.testing.assert_array_equal(out[0][1], out[1][1])
    assert out[0][2] == out[1][2]


@pytest.mark.gpu
def test_grid_count_limits():
    sc = scenes.water_cube(n_histories=1, n=4, bins=2)
    tables = M.Tables(sc.materials, e_max=sc.e_max)
    g = (sc.ids, sc.spacing, sc.origin)
    with pytest.raises(N.MidsxError) as e:
        M.Phantom.from_grids(tables, sc.domain, sc.background, [g] * 17)
    assert e.value.status == N.INVALID_ARG
    ph = M.Phantom.from_grids(tables, sc.domain, sc.background, [g] * 16)
    assert ph.n_voxels == 16 * sc.ids.size
