"""GPU parity tests: the CUDA path through the C ABI against the CPU oracle.

* table indexing is bit-exact (every lookup class, nodes, their float neighbours,
  midpoints, spectrum energies, random energies);
* the samplers (Rayleigh RITA, Compton Kahn + S(x), free path) draw the same numbers as the
  oracle on the same Philox streams (FP64) and the same distribution (KS) in FP32, and
  match the analytic densities;
* transport: per-history deposits of the FP64 kernel equal the oracle's on the same
  streams; totals within 0.5%; per-voxel and per-bin chi-square against an independent
  oracle run (mt19937 streams); scalar tallies;
* the mixed path (FP32 + 64-bit fixed point) against FP64 on identical streams, and its
  determinism (bit-identical repeat and split runs);
* the reference's own half-value-layer results;
* error statuses.
"""
import math

import numpy as np
import pytest

import midsx_gb300 as M
import oracle
from midsx_gb300 import native as N
from midsx_gb300 import scenes

pytestmark = pytest.mark.gpu


# ------------------------------------------------------------------------ helpers ---
def ks_2samp(a, b):
    from scipy.stats import ks_2samp as ks
    return ks(a, b).pvalue


def chi_voxels(s_a, q_a, s_b, q_b, frac=0.01):
    """z-scores of voxels above frac x max, with per-voxel variance estimated from the
    deposit sums of squares of each run (each run's sum is a compound sum of deposits)."""
    m = max(s_a.max(), s_b.max())
    sel = (s_a > frac * m) | (s_b > frac * m)
    var = q_a[sel] + q_b[sel]
    z = (s_a[sel] - s_b[sel]) / np.sqrt(np.maximum(var, 1e-300))
    return z


@pytest.fixture(scope="module")
def cube():
    sc = scenes.water_cube(n_histories=200_000, n=50, bins=50)
    objs = sc.build()
    return sc, objs


# ----------------------------------------------------------------- table indexing ---
def test_table_indices_bit_exact():
    mats = [scenes.AIR, scenes.SOFT_TISSUE, scenes.CORTICAL_BONE, scenes.LEAD]
    tables = M.Tables(mats, e_max=150e3)
    # the device's bucketed searches against full searches of the same (product) arrays; the
    # oracle's own build has the same node grids (tests/test_oracle.py)
    blob = tables.host
    rng = np.random.default_rng(1)
    spec_e, _ = scenes.kramers_spectrum(100.0)
    for m in range(len(mats)):
        t = blob.blob.mat[m]
        nodes = [blob.array(blob.blob.majorant.x, blob.blob.majorant.n), blob.array(t.total.x, t.total.n),
                 blob.array(t.sfunc.x, t.sfunc.n), blob.array(t.coh.knot_e, t.coh.n_ctrl + t.coh.degree + 1),
                 blob.array(t.incoh.knot_e, t.incoh.n_ctrl + t.incoh.degree + 1),
                 blob.array(t.rita.energy, t.rita.n_energy)]
        e = np.concatenate(nodes)
        e = e[np.isfinite(e) & (e > 0)]
        e = np.concatenate([e, np.nextafter(e, 0), np.nextafter(e, np.inf), (e[1:] + e[:-1]) / 2, spec_e,
                            np.exp(rng.uniform(np.log(1.0), np.log(1.5e5), 1_000_000))])
        e = e[(e > 0) & (e <= 1.5e5)]
        gpu = M.table_index(tables, m, e)
        cpu = oracle.table_index(blob, m, e)
        mism = np.nonzero(np.any(gpu != cpu, axis=1))[0]
        assert mism.size == 0, (m, e[mism[:5]], gpu[mism[:5]], cpu[mism[:5]])


# ---------------------------------------------------------------------- samplers ---
@pytest.mark.parametrize("energy", [20e3, 60e3, 79433.0, 120e3])
@pytest.mark.parametrize("mat", [scenes.WATER, scenes.CORTICAL_BONE, scenes.LEAD])
def test_samplers_match_oracle_streams(energy, mat):
    tables = M.Tables([mat], e_max=150e3)
    n = 200_000
    for kind in ("rayleigh", "compton", "freepath"):
        g = M.sample(tables, kind, 0, energy, n, seed=9, precision="fp64")
        c = oracle.sample(oracle.tables_like(tables), kind, 0, energy, n, seed=9)
        if kind == "compton":
            for a, b in zip(g, c):
                assert np.mean(np.abs(a - b) < 1e-9) > 0.999
        else:
            assert np.mean(np.abs(g - c) < 1e-9) > 0.999, kind
        g32 = M.sample(tables, kind, 0, energy, n, seed=9, precision="mixed")
        a32 = g32[0] if kind == "compton" else g32
        b64 = c[0] if kind == "compton" else c
        assert ks_2samp(a32, b64) > 1e-3, kind
        # same streams: FP32 draws are the FP64 draws rounded to 24 bits
        assert np.mean(np.abs(a32 - b64) < 1e-4 * max(1.0, np.abs(b64).max())) > 0.99, kind


def test_rayleigh_matches_analytic_density():
    """KS of the device RITA sampler against (1 + mu^2) F(x)^2 integrated numerically
    (the reference's own by-eye check: tests/distributions/distributions.cpp, Al 60 keV),
    at a table energy node, where RITA has no energy interpolation."""
    from scipy.stats import kstest
    tables = M.Tables([scenes.ALUMINIUM], e_max=150e3)
    blob = oracle.tables_like(tables)  # the analytic density from the oracle's own tables
    r = blob.blob.mat[0].rita
    E = blob.array(r.energy, r.n_energy)
    e_node = float(E[np.argmin(np.abs(E - 60e3))])
    mu = M.sample(tables, "rayleigh", 0, e_node, 400_000, seed=3, precision="fp64")
    alpha = 0.51099895000E6 / (math.sqrt(2.0) * 4.135667662e-15 * 299792458E2 * 1E8)
    s = np.linspace(0, math.sqrt(2), 200001)
    grid = 1 - s * s
    f = blob.eval(0, "ffactor", alpha * e_node / 0.51099895000E6 * np.sqrt(1 - grid))
    f = np.where(np.isnan(f), blob.eval(0, "ffactor", np.zeros(1))[0], f)
    pdf = (1 + grid ** 2) * f * f * 2 * s
    cdf_s = np.concatenate([[0], np.cumsum((pdf[1:] + pdf[:-1]) / 2 * np.diff(s))])
    cdf_s /= cdf_s[-1]
    # CDF in mu: P(MU <= m) = 1 - P(S <= sqrt(1 - m))
    def cdf(m):
        return 1 - np.interp(np.sqrt(np.clip(1 - m, 0, 2)), s, cdf_s)
    # the reference's RITA rows stop short of 1 (Simpson normalisation), leaving an atom at
    # mu = 1; compare the continuous part
    cont = mu[mu < 1.0]
    y_last = blob.array(r.y, r.n_rows)[blob.iarray(r.row_start, r.n_energy + 1)[np.argmin(np.abs(E - 60e3)) + 1] - 1]
    assert abs(np.mean(mu == 1.0) - max(0.0, 1 - y_last)) < 3e-3
    assert kstest(cont, lambda m: np.minimum(cdf(m) / max(y_last, 1e-12), 1.0)).pvalue > 1e-3


def test_compton_matches_klein_nishina_times_sfunc():
    from scipy.stats import kstest
    tables = M.Tables([scenes.WATER], e_max=150e3)
    blob = oracle.tables_like(tables)  # the analytic density from the oracle's own tables
    E = 80e3
    k = E / 0.51099895000E6
    mu, _ = M.sample(tables, "compton", 0, E, 400_000, seed=4, precision="fp64")
    alpha = 0.51099895000E6 / (math.sqrt(2.0) * 4.135667662e-15 * 299792458E2 * 1E8)
    grid = np.linspace(-1, 1, 400001)
    r = 1 / (1 + k * (1 - grid))
    kn = r * r * (r + 1 / r - (1 - grid * grid))
    S = blob.eval(0, "sfunc", np.maximum(alpha * k * np.sqrt(1 - grid), 1e-300))
    S = np.nan_to_num(S)
    pdf = kn * S
    cdf = np.concatenate([[0], np.cumsum((pdf[1:] + pdf[:-1]) / 2 * np.diff(grid))])
    cdf /= cdf[-1]
    assert kstest(mu, lambda m: np.interp(m, grid, cdf)).pvalue > 1e-3


# --------------------------------------------------------------------- transport ---
def test_fp64_histories_equal_oracle_on_same_streams(cube):
    sc, (tables, ph, src, tl) = cube
    n = 100_000
    g = M.trace_deposits(tables, ph, src, n, seed=21, precision="fp64")
    o = oracle.run(oracle.tables_like(tables), n=n, seed=21, history=True, dose=False, **sc.oracle_kwargs())["history_deposit"]
    same = np.abs(g - o) <= 1e-9 * np.maximum(1.0, np.abs(o))
    assert same.mean() > 0.999, same.mean()
    assert abs(g.sum() - o.sum()) / o.sum() < 1e-3


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_water_cube_against_independent_oracle(cube, precision):
    """Per-voxel dose chi-square, totals within 0.5%, and the binned exit-plane tally,
    against the oracle run with the reference's own generator (mt19937, independent)."""
    sc, (tables, ph, src, tl) = cube
    n = 400_000
    tl.reset()
    M.run(tables, ph, src, tl, n, seed=5, precision=precision)
    st = tl.stats()
    d = tl.dose()
    be, bc = tl.binned(0)
    o = oracle.run(oracle.tables_like(tables), n=n, seed=5, rng=oracle.RNG_MT19937, **sc.oracle_kwargs())
    so = o["stats"]
    assert st["histories"] == n
    bal = st["deposited_grid"] + st["deposited_background"] + st["escaped_energy"]
    assert bal == pytest.approx(st["source_energy"], rel=1e-6)
    assert abs(st["deposited_grid"] - so["deposited_grid"]) / so["deposited_grid"] < 0.005
    assert abs(st["escaped_energy"] - so["escaped_energy"]) / so["escaped_energy"] < 0.005
    oe, oc = o["binned"][0]
    # exit-plane total: within 0.5 %, or within 4 sigma where the sample cannot resolve 0.5 %
    # (at 4e5 histories the two runs' totals differ by ~0.45 % at one sigma); sigma from the
    # bins' Poisson-compound variances, tot^2 / count per bin
    cg, co = bc.sum(axis=2).ravel(), oc.sum(axis=2).ravel()
    tg, to = be.sum(axis=2).ravel(), oe.sum(axis=2).ravel()
    var = (tg[cg > 0] ** 2 / cg[cg > 0]).sum() + (to[co > 0] ** 2 / co[co > 0]).sum()
    assert abs(be.sum() - oe.sum()) < max(0.005 * oe.sum(), 4 * np.sqrt(var)), (be.sum(), oe.sum(), np.sqrt(var))
    z = chi_voxels(d["sum"].ravel(), d["sumsq"].ravel(), o["dose"]["sum"].ravel(), o["dose"]["sumsq"].ravel())
    assert z.size > 50
    assert np.mean(np.abs(z) > 3) < 0.01, np.mean(np.abs(z) > 3)
    # chi-square per voxel: mean z^2 is 1 within its own sampling error sqrt(2 / n_voxels)
    # (the deposit-based variance is conservative, so a mean well below 1 is allowed)
    assert np.mean(z * z) < 1 + 4 * np.sqrt(2 / z.size), np.mean(z * z)
    # detector bins (primary + scattered), Poisson-compound variance from counts
    tot_g, tot_o = be.sum(axis=2).ravel(), oe.sum(axis=2).ravel()
    cnt_g, cnt_o = bc.sum(axis=2).ravel(), oc.sum(axis=2).ravel()
    sel = (cnt_g + cnt_o) > 200
    zb = (tot_g[sel] - tot_o[sel]) / np.sqrt((tot_g[sel] ** 2 / np.maximum(cnt_g[sel], 1)) +
                                              (tot_o[sel] ** 2 / np.maximum(cnt_o[sel], 1)))
    assert np.mean(np.abs(zb) > 4) < 0.01


def test_mixed_against_fp64_identical_streams(cube):
    sc, (tables, ph, src, tl) = cube
    n = 200_000
    out = {}
    for p in ("fp64", "mixed"):
        tl.reset()
        M.run(tables, ph, src, tl, n, seed=8, precision=p)
        out[p] = (tl.stats(), tl.dose())
    s64, d64 = out["fp64"]
    s32, d32 = out["mixed"]
    assert abs(s32["deposited_grid"] - s64["deposited_grid"]) / s64["deposited_grid"] < 0.005
    z = chi_voxels(d32["sum"].ravel(), d32["sumsq"].ravel(), d64["sum"].ravel(), d64["sumsq"].ravel())
    assert np.mean(np.abs(z) > 3) < 0.003  # identical streams: far inside the MC noise
    g64 = M.trace_deposits(tables, ph, src, 50_000, seed=8, precision="fp64")
    g32 = M.trace_deposits(tables, ph, src, 50_000, seed=8, precision="mixed")
    assert np.mean(np.abs(g32 - g64) <= 1e-3 * np.maximum(1.0, g64)) > 0.97


def test_mixed_is_deterministic_and_split_invariant(cube):
    """64-bit fixed-point tallies are order independent: a repeat run and a run split into
    two history ranges give bit-identical tallies (a thread-order race would show here)."""
    sc, (tables, ph, src, tl) = cube
    n = 100_000
    res = []
    for parts in ([(0, n)], [(0, n)], [(0, n // 3), (n // 3, n - n // 3)]):
        tl.reset()
        for first, cnt in parts:
            M.run(tables, ph, src, tl, cnt, seed=13, first=first, precision="mixed")
        d = tl.dose()
        be, bc = tl.binned(0)
        st = tl.stats()
        res.append((d["sum"].copy(), d["sumsq"].copy(), d["count"].copy(), be.copy(), bc.copy(), st))
    for r in res[1:]:
        for a, b in zip(res[0][:5], r[:5]):
            np.testing.assert_array_equal(a, b)
        for k in ("steps", "voxel_fetches", "photo", "coherent", "incoherent", "deposited_grid"):
            assert res[0][5][k] == r[5][k]


def test_scalar_tallies_match_oracle_streams():
    """Disc, rectangle and axis-aligned cuboid tallies (all quantities and classes) against
    the oracle on the same Philox streams."""
    sc = scenes.water_cube(n_histories=1, n=40, bins=8)
    specs = [dict(kind="disc", center=(10, 10, 15), normal=(0, 0, 1), radius=3.0),
             dict(kind="rect", corner=(5, 5, 15), edge1=(10, 0, 0), edge2=(0, 10, 0)),
             dict(kind="cuboid", min=(8, 8, 5), max=(12, 12, 9)),
             dict(kind="cuboid", min=(0, 0, 0), max=(20, 20, 4)),
             dict(kind="binned", corner=(5, 5, 15), edge1=(10, 0, 0), edge2=(0, 10, 0), nu=8, nv=8)]
    tables = M.Tables(sc.materials, e_max=sc.e_max)
    ph = M.Phantom(tables, sc.domain, sc.spacing, sc.origin, sc.ids, sc.background)
    src = M.Source(position=(10, 10, 0), direction=("disc", (10, 10, 5), (0, 0, 1), 4.0), energy=60e3)
    tl = M.Tallies(ph, specs, N.DOSE_OFF)
    n = 200_000
    M.run(tables, ph, src, tl, n, seed=17, precision="fp64")
    kw = sc.oracle_kwargs()
    kw.update(specs=specs, source=dict(position=(10, 10, 0), direction=("disc", (10, 10, 5), (0, 0, 1), 4.0),
                                       energy=60e3))
    o = oracle.run(oracle.tables_like(tables), n=n, seed=17, dose=False, **kw)
    for i in range(4):
        g = tl.scalar(i)
        c = o["scalar"][i]
        counts = np.r_[g[0:24:3], g[24:32]]
        ocounts = np.r_[c[0:24:3], c[24:32]]
        assert np.all(np.abs(counts - ocounts) <= np.maximum(3, 2e-3 * ocounts)), (i, counts, ocounts)
        sums = g[1:24:3]
        osums = c[1:24:3]
        assert np.all(np.abs(sums - osums) <= 2e-3 * np.abs(osums) + 1e-6 * np.abs(osums).max()), i
    be, bc = tl.binned(4)
    oe, oc = o["binned"][4]
    assert np.all(np.abs(bc - oc) <= np.maximum(3, 2e-3 * oc))


def test_cone_beam_crop_against_oracle():
    """A 64x64x32 crop of the heterogeneous cone-beam phantom (four materials, Kramers
    spectrum, disc cone source): totals and voxel chi-square against the oracle."""
    sc = scenes.cone_beam_dose(n_histories=1, shape=(32, 64, 64), spacing=0.1, seed=2)
    tables, ph, src, tl = sc.build()
    n = 300_000
    for p in ("fp64", "mixed"):
        tl.reset()
        M.run(tables, ph, src, tl, n, seed=31, precision=p)
        st = tl.stats()
        d = tl.dose()
        o = oracle.run(oracle.tables_like(tables), n=n, seed=32, rng=oracle.RNG_MT19937, **sc.oracle_kwargs())
        so = o["stats"]
        assert abs(st["deposited_grid"] - so["deposited_grid"]) / so["deposited_grid"] < 0.01
        assert abs(st["steps"] - so["steps"]) / so["steps"] < 0.005
        z = chi_voxels(d["sum"].ravel(), d["sumsq"].ravel(), o["dose"]["sum"].ravel(), o["dose"]["sumsq"].ravel())
        assert np.mean(np.abs(z) > 3) < 0.015, (p, np.mean(np.abs(z) > 3))


# ------------------------------------------------------------------ golden HVL ---
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["30keV", "100keV"])
def test_gpu_reproduces_reference_hvl(golden, case, precision):
    sc = golden["scene"]
    tables = M.Tables([scenes.AIR, scenes.ALUMINIUM], e_max=150e3)
    n = 2_000_000
    src = M.Source(position=sc["source"]["position"],
                   direction=("disc", sc["source"]["disc_center"], sc["source"]["disc_normal"],
                              sc["source"]["disc_radius"]), energy=float(case.replace("keV", "")) * 1e3)
    counts = {}
    for kind in ("0", "hvl", "qvl"):
        if kind == "0":
            ids, spacing = np.full((1, 1, 1), scenes.AIR, np.uint8), (4, 4, 1e-4)
        else:
            s = golden["cases"][case]["slab_" + kind]
            ids, spacing = np.full((s["dims"][2], 1, 1), s["material_id"], np.uint8), s["spacing_cm"]
        ph = M.Phantom(tables, sc["domain"], spacing, sc["slab_origin"], ids, scenes.AIR)
        tl = M.Tallies(ph, [dict(kind="disc", **sc["disc_tally"])], N.DOSE_OFF)
        M.run(tables, ph, src, tl, n, seed=100 + len(counts), precision=precision)
        counts[kind] = tl.scalar(0)[0]
    ref = golden["cases"][case]
    for kind in ("hvl", "qvl"):
        r = counts[kind] / counts["0"]
        r_ref = ref["AK_" + kind]["mean"] / ref["AK_0"]["mean"]
        pa, pb = counts[kind] / n, counts["0"] / n
        sig = r * math.sqrt((1 - pa) / (n * pa) + (1 - pb) / (n * pb))
        assert abs(r - r_ref) < 4 * math.hypot(sig, 1e-4 * r_ref), (kind, r, r_ref)


# ---------------------------------------------------------------- error statuses ---
def test_error_statuses():
    tables = M.Tables([scenes.AIR, scenes.WATER], e_max=70e3)
    ids = np.full((4, 4, 4), scenes.WATER, np.uint8)
    ph = M.Phantom(tables, (10, 10, 10), (1, 1, 1), (3, 3, 3), ids, scenes.AIR)
    with pytest.raises(N.MidsxError) as e:
        M.Phantom(tables, (10, 10, 10), (1, 1, 1), (3, 3, 3), np.full((4, 4, 4), scenes.LEAD, np.uint8), scenes.AIR)
    assert e.value.status == N.NOT_FOUND
    hot = M.Source(position=(5, 5, 0), direction=("beam", (5, 5, 10)), energy=100e3)
    tl = M.Tallies(ph, [], N.DOSE_SUM)
    with pytest.raises(N.MidsxError) as e:
        M.run(tables, ph, hot, tl, 100, seed=1)
    assert e.value.status == N.TABLE_RANGE
    src = M.Source(position=(5, 5, 0), direction=("beam", (5, 5, 10)), energy=60e3)
    M.run(tables, ph, src, tl, 10_000, seed=1, max_steps=2)
    with pytest.raises(N.MidsxError) as e:
        tl.stats()
    assert e.value.status == N.STEP_CAP
    st = tl.stats(allow_cap=True)
    assert st["step_cap_hits"] > 0 and st["histories"] == 10_000
    with pytest.raises(N.MidsxError) as e:
        M.Source(position=(0, 0, 0), direction=("rect", (0, 0, 1), (1, 0, 0), (1, 1, 0)), energy=60e3)
    assert e.value.status == N.INVALID_ARG
    with pytest.raises(N.MidsxError):
        M.run(tables, ph, src, tl, 10, seed=1, precision="fp64")  # tallies hold mixed results


def test_fp32_lookups_finite_on_grid_nodes_closer_than_float_resolution():
    """Merged energy grids hold node pairs a few meV apart whose log10 energies round to one
    float: in FP32 such an interval has zero width.  A majorant recomputing its slope there in
    FP32 was infinite, and the photon took zero-length steps until the step cap (one history in
    ~5e8 of the cone-beam workload).  The FP32 tables carry slopes computed in FP64: free paths
    sampled at those nodes are finite and equal the FP64 ones on the same streams, and that
    history now ends after a normal number of steps."""
    sc = scenes.cone_beam_dose(n_histories=1)
    tables, ph, src, tl = sc.build()
    blob = tables.host
    mj = blob.blob.majorant
    x, lx = blob.array(mj.x, mj.n), blob.array(mj.lx, mj.n)
    fx = lx.astype(np.float32)
    bad = np.nonzero((fx[1:] <= fx[:-1]) & (lx[1:] > lx[:-1]) & np.isfinite(lx[:-1]))[0]
    e = x[bad][(x[bad] > 1e3) & (x[bad] < 8e4)]
    assert e.size > 20
    for E in e[:: max(1, e.size // 40)]:
        E32 = float(np.float32(E))
        s32 = M.sample(tables, "freepath", 0, E32, 64, seed=5, precision="mixed")
        s64 = M.sample(tables, "freepath", 0, E32, 64, seed=5, precision="fp64")
        assert np.all(np.isfinite(s32)) and np.all(s32 > 0), E
        np.testing.assert_allclose(s32, s64, rtol=2e-4, atol=1e-5 * s64.mean())
    tl.reset()
    M.run(tables, ph, src, tl, 1, seed=1, first=20200762447, precision="mixed")
    st = tl.stats()
    assert st["step_cap_hits"] == 0 and st["steps"] < 1000
