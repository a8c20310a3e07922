"""Parity of the CUDA path with the CPU oracle at the benchmark configurations' own sizes.

* Water cube (100^3 water voxels at 1 mm in a 20 cm air box, 60 keV pencil beam, 100 x 100
  exit-plane bins, 1e6 histories, seed 1): the plain FP64 kernel equals the oracle on the same
  Philox streams voxel by voxel, and both precisions agree with an independent oracle run
  (the reference's mt19937 generator): per-voxel chi-square over voxels above 1 % of the
  maximum, deposited and transmitted energy within 0.5 %, per-bin chi-square on the exit
  plane.  Reference loop: src/MIDSX/Core/physics_engine.cpp:17-79, run_simulation.cpp:6-41;
  exit-plane semantics: surface_tally.cpp:16-34.
* Cone-beam dose (the full 256 x 256 x 128 phantom at 0.5 mm, 80 kVp, 2e6 histories): both
  precisions against an independent oracle run - totals, Woodcock steps per history and the
  per-voxel chi-square.
* Radiography with lead (512 x 512 x 256 at 0.5 mm with sixteen 2 mm lead spheres, 100 kVp,
  512 x 512 detector at 100 cm): the FP64 kernel equals the oracle on the same Philox streams
  (detector images by scatter class), and both precisions agree with an independent oracle
  run on primary and scattered totals and on a 16 x 16 rebinned detector image
  (surface_quantity.cpp:49-63 classes).  No history reaches the step cap.

The oracle runs with its own tables (oracle/tables.py restates the reference's table
construction), so a table-build error of the product would show here as well.  Voxel
z-scores divide by history-based variances of each run's sum - on the device the batch method
with 256 batches (MIDSX_DOSE_BATCHES), in the oracle the exact per-history estimator - not by
the reference's per-deposit sigma (src/MIDSX/Core/quantity.cpp:37-45), and compare only
voxels (or blocks of voxels) holding at least 50 deposits in both runs, where a sum is close
to Gaussian.  The cone-beam phantom at 2e6 histories holds well under one deposit per 0.5 mm
voxel, so its chi-square runs on 16 x 16 x 8 mm blocks, with batch sums of the blocks
themselves (a history's deposits in neighbouring voxels are correlated).
"""
import numpy as np
import pytest

import midsx_gb300 as M
import oracle
from midsx_gb300 import native as N
from midsx_gb300 import scenes

BATCHES = 16       # same-stream comparison of the batch variance
GPU_BATCHES = 256  # the device's variance in the independent comparisons
MIN_DEPOSITS = 50

pytestmark = pytest.mark.gpu


def z_voxels(g, o, frac=0.01):
    """z-scores of the voxels above frac x the larger maximum with at least MIN_DEPOSITS
    deposits in both runs: device dose g (batch variance "var") against oracle dose o
    (per-history variance "var_hist")."""
    s_a, s_b = g["sum"].ravel(), o["sum"].ravel()
    m = max(s_a.max(), s_b.max())
    sel = ((s_a > frac * m) | (s_b > frac * m)) & (g["count"].ravel() >= MIN_DEPOSITS) & \
        (o["count"].ravel() >= MIN_DEPOSITS)
    v = g["var"].ravel()[sel] + o["var_hist"].ravel()[sel]
    return (s_a[sel] - s_b[sel]) / np.sqrt(np.maximum(v, 1e-300))


def assert_chi(z, beyond=0.01, label="", dof=GPU_BATCHES - 1):
    """Fewer than `beyond` of the z-scores past 3 sigma, and mean z^2 = 1 within 5 times its
    sampling error sqrt(2 / n) plus 4 / dof, the inflation of E[z^2] that a variance estimated
    from dof degrees of freedom brings (2 / dof for Gaussian batch sums, doubled for their
    skew)."""
    assert z.size > 50, (label, z.size)
    assert np.mean(np.abs(z) > 3) < beyond, (label, np.mean(np.abs(z) > 3))
    assert np.mean(z * z) < 1 + 5 * np.sqrt(2 / z.size) + 4.0 / dof, (label, np.mean(z * z))


def z_bins(e_a, c_a, e_b, c_b, min_count=100):
    """Per-bin z-scores of two binned energy images (compound-Poisson variance sum^2 / count
    for each), over bins holding at least min_count crossings in both."""
    sel = (c_a >= min_count) & (c_b >= min_count)
    va = e_a[sel] ** 2 / c_a[sel]
    vb = e_b[sel] ** 2 / c_b[sel]
    return (e_a[sel] - e_b[sel]) / np.sqrt(va + vb)


def rebin(img, k):
    ny, nx = img.shape[:2]
    return img.reshape(ny // k, k, nx // k, k, *img.shape[2:]).sum(axis=(1, 3))


# ------------------------------------------------------------------- water cube ---
@pytest.fixture(scope="module")
def cube():
    sc = scenes.water_cube()  # 100^3 at 1 mm, 100 x 100 bins
    assert sc.ids.shape == (100, 100, 100) and sc.specs[0]["nu"] == 100
    sc.dose_mode = N.DOSE_BATCHES
    objs = sc.build()
    blob = oracle.tables_for(sc)
    return sc, objs, blob


def test_water_cube_fp64_equals_oracle_on_same_streams(cube):
    sc, (tables, ph, src, tl), blob = cube
    n = 1_000_000
    tl.reset()
    M.run(tables, ph, src, tl, n, seed=1, precision="fp64", variance_batches=BATCHES)
    st = tl.stats()
    d = tl.dose()
    be, bc = tl.binned(0)
    o = oracle.run_batches(blob, BATCHES, n=n, seed=1, **sc.oracle_kwargs())
    so = o["stats"]
    assert st["histories"] == so["histories"] == n
    assert st["step_cap_hits"] == so["step_cap_hits"] == 0
    # same streams: every count equal but for the rare history that meets a decision within
    # rounding of the two builds' tables
    for k in ("steps", "photo", "coherent", "incoherent"):
        assert abs(st[k] - so[k]) <= 1e-4 * so[k] + 2, k
    assert st["deposited_grid"] == pytest.approx(so["deposited_grid"], rel=1e-4)
    assert st["escaped_energy"] == pytest.approx(so["escaped_energy"], rel=1e-4)
    g, c = d["sum"].ravel(), o["dose"]["sum"].ravel()
    same = np.abs(g - c) <= 1e-9 * np.maximum(1.0, np.abs(c))
    assert same.mean() > 0.999, same.mean()
    # the same batches on the same streams: the batch variances agree as the sums do
    vg, vc = d["var"].ravel(), o["dose"]["var"].ravel()
    assert np.mean(np.abs(vg - vc) <= 1e-6 * np.maximum(vc, 1e-30) + 1e-9 * vc.max()) > 0.999
    oe, oc = o["binned"][0]
    assert np.mean(bc == oc) > 0.999
    assert be.sum() == pytest.approx(oe.sum(), rel=1e-4)


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_water_cube_against_independent_oracle_full_size(cube, precision):
    sc, (tables, ph, src, tl), blob = cube
    n = 1_000_000
    tl.reset()
    M.run(tables, ph, src, tl, n, seed=1, precision=precision, variance_batches=GPU_BATCHES)
    st = tl.stats()
    d = tl.dose()
    assert d["batches"] == GPU_BATCHES
    be, bc = tl.binned(0)
    o = oracle.run(blob, n=n, seed=1, rng=oracle.RNG_MT19937, **sc.oracle_kwargs())
    so = o["stats"]
    assert st["step_cap_hits"] == 0
    bal = st["deposited_grid"] + st["deposited_background"] + st["escaped_energy"]
    assert bal == pytest.approx(st["source_energy"], rel=1e-6)
    assert abs(st["deposited_grid"] - so["deposited_grid"]) / so["deposited_grid"] < 0.005
    assert abs(st["escaped_energy"] - so["escaped_energy"]) / so["escaped_energy"] < 0.005
    oe, oc = o["binned"][0]
    # transmitted energy on the exit plane (all classes) within 0.5 %
    assert abs(be.sum() - oe.sum()) / oe.sum() < 0.005
    assert_chi(z_voxels(d, o["dose"]), label="voxels")
    zb = z_bins(be.sum(axis=2).ravel(), bc.sum(axis=2).ravel(), oe.sum(axis=2).ravel(), oc.sum(axis=2).ravel())
    assert_chi(zb, label="exit-plane bins", dof=1e9)


# -------------------------------------------------------------- cone-beam dose ---
CONE_BLOCK = (16, 32, 32)  # (z, y, x) voxels of 0.5 mm: 8 x 16 x 16 mm blocks
CONE_BATCHES = 32


def blocks(a, k=CONE_BLOCK):
    a = np.asarray(a).reshape(128, 256, 256)
    return a.reshape(128 // k[0], k[0], 256 // k[1], k[1], 256 // k[2], k[2]).sum(axis=(1, 3, 5)).ravel()


@pytest.fixture(scope="module")
def cone():
    sc = scenes.cone_beam_dose(n_histories=1)
    assert sc.ids.shape == (128, 256, 256)
    objs = sc.build()
    return sc, objs, oracle.tables_for(sc)


def test_cone_beam_full_phantom_fp64_equals_oracle_on_same_streams(cone):
    sc, (tables, ph, src, tl), blob = cone
    n = 2_000_000
    tl.reset()
    M.run(tables, ph, src, tl, n, seed=43, precision="fp64")
    st, d = tl.stats(), tl.dose()
    o = oracle.run(blob, n=n, seed=43, **sc.oracle_kwargs())
    so = o["stats"]
    for k in ("steps", "voxel_fetches", "photo", "coherent", "incoherent"):
        assert abs(st[k] - so[k]) <= 1e-4 * so[k] + 2, k
    g, c = d["sum"].ravel(), o["dose"]["sum"].ravel()
    hit = (g > 0) | (c > 0)
    same = np.abs(g[hit] - c[hit]) <= 1e-9 * np.maximum(1.0, c[hit])
    assert hit.sum() > 100_000 and same.mean() > 0.999, (hit.sum(), same.mean())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_cone_beam_full_phantom_against_independent_oracle(cone, precision):
    sc, (tables, ph, src, tl), blob = cone
    n, B = 2_000_000, CONE_BATCHES
    tl.reset()
    # the device's batch sums of each block: B runs over consecutive history ranges
    prev, gsums, first = 0.0, [], 0
    for b in range(B):
        M.run(tables, ph, src, tl, n // B, seed=41, first=first, precision=precision)
        first += n // B
        cur = blocks(tl.dose()["sum"])
        gsums.append(cur - prev)
        prev = cur
    st = tl.stats()
    o = oracle.run_batches(blob, B, n=n, seed=42, rng=oracle.RNG_MT19937, reduce=blocks, **sc.oracle_kwargs())
    so = o["stats"]
    assert st["step_cap_hits"] == 0 and so["step_cap_hits"] == 0
    assert abs(st["deposited_grid"] - so["deposited_grid"]) / so["deposited_grid"] < 0.005
    assert abs(st["escaped_energy"] - so["escaped_energy"]) / so["escaped_energy"] < 0.005
    assert abs(st["steps"] - so["steps"]) / so["steps"] < 0.005
    assert abs(st["voxel_fetches"] - so["voxel_fetches"]) / so["voxel_fetches"] < 0.005
    G, O = np.stack(gsums), o["dose"]["batch_sums"]
    vg = B / (B - 1) * ((G - G.mean(axis=0)) ** 2).sum(axis=0)
    vo = o["dose"]["var"]
    sg, so_ = G.sum(axis=0), O.sum(axis=0)
    cg, co = blocks(tl.dose()["count"]), blocks(o["dose"]["count"])
    sel = ((sg > 0.01 * sg.max()) | (so_ > 0.01 * so_.max())) & (cg >= 32 * MIN_DEPOSITS) & (co >= 32 * MIN_DEPOSITS)
    z = (sg[sel] - so_[sel]) / np.sqrt(vg[sel] + vo[sel])
    assert_chi(z, beyond=0.012, label="blocks", dof=2 * (B - 1))


# ----------------------------------------------------------- radiography, lead ---
@pytest.fixture(scope="module")
def radiograph():
    sc = scenes.radiography(n_histories=1)
    assert sc.ids.shape == (256, 512, 512) and int((sc.ids == scenes.LEAD).sum()) > 0
    objs = sc.build()
    blob = oracle.tables_for(sc)
    return sc, objs, blob


def test_radiography_fp64_equals_oracle_on_same_streams(radiograph):
    sc, (tables, ph, src, tl), blob = radiograph
    n = 20_000
    tl.reset()
    M.run(tables, ph, src, tl, n, seed=3, precision="fp64")
    st = tl.stats()
    be, bc = tl.binned(0)
    o = oracle.run(blob, n=n, seed=3, dose=False, **sc.oracle_kwargs())
    so = o["stats"]
    oe, oc = o["binned"][0]
    assert st["step_cap_hits"] == 0 and so["step_cap_hits"] == 0
    assert abs(st["steps"] - so["steps"]) <= 1e-3 * so["steps"]
    # detector counts by scatter class: the same photons in the same bins
    for cls in range(4):
        assert np.abs(bc[..., cls] - oc[..., cls]).sum() <= 1e-3 * oc[..., cls].sum() + 4, cls
        assert be[..., cls].sum() == pytest.approx(oe[..., cls].sum(), rel=2e-3, abs=1e-6), cls


@pytest.fixture(scope="module")
def radiograph_oracle(radiograph):
    """One independent oracle run (mt19937) shared by both precisions: 1e5 histories at
    ~17.5k Woodcock steps each."""
    sc, _, blob = radiograph
    return oracle.run(blob, n=100_000, seed=12, rng=oracle.RNG_MT19937, dose=False, **sc.oracle_kwargs())


@pytest.mark.parametrize("precision", ["fp64", "mixed"])
def test_radiography_against_independent_oracle(radiograph, radiograph_oracle, precision):
    sc, (tables, ph, src, tl), blob = radiograph
    n_gpu = 1_000_000 if precision == "fp64" else 4_000_000
    n_cpu = 100_000
    tl.reset()
    M.run(tables, ph, src, tl, n_gpu, seed=11, precision=precision)
    st = tl.stats()
    be, bc = tl.binned(0)
    o = radiograph_oracle
    so = o["stats"]
    oe, oc = o["binned"][0]
    assert st["step_cap_hits"] == 0 and so["step_cap_hits"] == 0
    # Woodcock steps per history: the same algorithm against the same (lead) majorant
    assert abs(st["steps"] / n_gpu - so["steps"] / n_cpu) / (so["steps"] / n_cpu) < 0.01
    # primary and scattered totals per history, within 4 sigma of the two samples (the
    # oracle's 1e5 histories dominate) - counts per history are binomial-like
    for name, cls in (("primary", [0]), ("scatter", [1, 2, 3])):
        cg, co = bc[..., cls].sum() / n_gpu, oc[..., cls].sum() / n_cpu
        eg, eo = be[..., cls].sum() / n_gpu, oe[..., cls].sum() / n_cpu
        sig_c = np.sqrt(cg / n_gpu + co / n_cpu)
        assert abs(cg - co) < 4 * sig_c, (name, cg, co, sig_c)
        assert abs(eg - eo) / eo < 4 * sig_c / co + 1e-3, (name, eg, eo)
    # rebinned images, per class group, per history: 16 x 16 (32 x 32 detector bins each) for
    # the primaries, 8 x 8 for the scattered photons (fewer)
    for cls, k in (([0], 32), ([1, 2, 3], 64)):
        ig = rebin(be[..., cls].sum(axis=2), k).ravel() / n_gpu
        cg = rebin(bc[..., cls].sum(axis=2), k).ravel()
        io = rebin(oe[..., cls].sum(axis=2), k).ravel() / n_cpu
        co = rebin(oc[..., cls].sum(axis=2), k).ravel()
        sel = (cg >= MIN_DEPOSITS) & (co >= MIN_DEPOSITS)
        z = (ig[sel] - io[sel]) / np.sqrt(ig[sel] ** 2 / cg[sel] + io[sel] ** 2 / co[sel])
        assert z.size > 10, (cls, z.size)
        assert np.mean(np.abs(z) > 3) < 0.02, (cls, np.mean(np.abs(z) > 3))
        assert np.mean(z * z) < 1 + 5 * np.sqrt(2 / z.size), (cls, np.mean(z * z))


# ------------------------------------------------------------- isotropic source ---
def test_isotropic_source_against_oracle():
    """IsotropicDirectionality (src/MIDSX/Core/source.cpp:62-70: theta ~ U[0, pi],
    phi ~ U[0, 2 pi), the reference's definition): a point source inside a water cube, FP64
    per-history deposits equal to the oracle's on the same streams, scalar cuboid tallies
    and the dose against an independent oracle run."""
    ids = np.full((40, 40, 40), scenes.WATER, np.uint8)
    source = dict(position=(10, 10, 10), direction=("isotropic",), energy=50e3)
    sc = scenes.Scene("isotropic_point_in_water", [scenes.AIR, scenes.WATER], (20, 20, 20), (0.1, 0.1, 0.1),
                      (8, 8, 8), ids, scenes.AIR, source,
                      [dict(kind="cuboid", min=(8, 8, 8), max=(10, 12, 12)),
                       dict(kind="disc", center=(10, 10, 19), normal=(0, 0, 1), radius=5.0)], N.DOSE_BATCHES, 1, 100e3)
    tables, ph, src, tl = sc.build()
    blob = oracle.tables_for(sc)
    n = 200_000
    g = M.trace_deposits(tables, ph, src, n, seed=2, precision="fp64")
    o = oracle.run(blob, n=n, seed=2, history=True, dose=False, **sc.oracle_kwargs())["history_deposit"]
    assert np.mean(np.abs(g - o) <= 1e-9 * np.maximum(1.0, o)) > 0.999
    for precision in ("fp64", "mixed"):
        tl.reset()
        M.run(tables, ph, src, tl, n, seed=3, precision=precision, variance_batches=GPU_BATCHES)
        d = tl.dose()
        oo = oracle.run(blob, n=n, seed=4, rng=oracle.RNG_MT19937, **sc.oracle_kwargs())
        for t in (0, 1):
            gs, os_ = tl.scalar(t), oo["scalar"][t]
            # photons counted (all classes): Poisson, within 4 sigma
            a, b = gs[24:28].sum(), os_[24:28].sum()
            assert abs(a - b) < 4 * np.sqrt(a + b) + 1, (precision, t, a, b)
            # first vector quantity (deposited energy of the cuboid, incident energy of the
            # disc) summed over classes, within 4 sigma from its sums of squares
            a, b = gs[1:12:3].sum(), os_[1:12:3].sum()
            va, vb = gs[2:12:3].sum(), os_[2:12:3].sum()
            assert abs(a - b) < 4 * np.sqrt(va + vb) + 1e-9 * abs(b), (precision, t, a, b)
        assert_chi(z_voxels(d, oo["dose"]), label=precision)


# -------------------------------------------------------- batch-method variance ---
@pytest.mark.parametrize("precision", ["mixed", "fp64"])
def test_batch_variance_equals_the_batches_computed_on_the_host(precision):
    """MIDSX_DOSE_BATCHES against the same batches run one by one into DOSE_FULL tallies,
    their sums differenced on the host: the same B / (B - 1) sum_b (S_b - S / B)^2 (exact
    integer batch sums in the mixed form; FP64 atomics round in thread order)."""
    sc = scenes.water_cube(n=30, bins=4)
    tables, ph, src, _ = sc.build()
    tb = M.Tallies(ph, (), N.DOSE_BATCHES)
    tf = M.Tallies(ph, (), N.DOSE_FULL)
    n, B = 120_000, 8
    M.run(tables, ph, src, tb, n, seed=9, first=5, precision=precision, variance_batches=B)
    got = tb.dose()
    assert got["batches"] == B
    prev, batch_sums, first = 0.0, [], 5
    for b in range(B):
        M.run(tables, ph, src, tf, n // B, seed=9, first=first, precision=precision)
        first += n // B
        cur = tf.dose()["sum"].ravel().copy()
        batch_sums.append(cur - prev)
        prev = cur
    S = np.stack(batch_sums)
    expect = B / (B - 1) * ((S - S.mean(axis=0)) ** 2).sum(axis=0)
    np.testing.assert_allclose(got["sum"].ravel(), prev, rtol=1e-12 if precision == "fp64" else 0)
    tol = 1e-12 if precision == "mixed" else 1e-8
    np.testing.assert_allclose(got["var"].ravel(), expect, rtol=tol, atol=tol * expect.max())
    # a second run adds one batch (each run closes at least one); a reset clears them
    M.run(tables, ph, src, tb, 1000, seed=10, precision=precision)
    assert tb.dose()["batches"] == B + 1
    tb.reset()
    assert "var" not in tb.dose()
