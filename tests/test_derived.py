"""Derived quantities (DerivedQuantity, src/MIDSX/Core/derived_quantities.cpp:3-68) over the
incident-energy spectra of disc / rect surface tallies, and the mass energy-absorption
coefficient they use.

* mu_en/rho from the built tables against the air table of the reference's data set
  (data/reference_set, TG-195 case 1 sheet, via tests/golden/hvl_reference.json) and against
  the transport's own Compton sampler;
* the spectrum form of getPrimaryFluence / getPrimaryAirKerma / getPrimarySpectrumAirKerma
  against the reference's algorithm on raw vectors (oracle/derived.py), on the oracle's
  transport of the half-value-layer scene, mono- and polyenergetic;
* the polyenergetic half-value layers of the reference's committed results (AK_hvl / AK_0,
  AK_qvl / AK_0 for the 30 kVp and 100 kVp spectra) through the spectrum air kerma;
* on the GPU: device spectra equal to the oracle's on the same Philox streams (FP64), the
  reference's ratios through the device path in both precisions, and the C++ program.
"""
import math

import numpy as np
import pytest

import midsx_gb300 as M
import oracle
from midsx_gb300 import derived as D
from midsx_gb300 import native as N
from midsx_gb300 import scenes
from oracle import derived as OD

MIDPOINTS = [(0.25 + 0.5 * k) * 1e3 for k in range(239)]  # the reference spectrum files' energies (eV)

# Relative allowance on the polyenergetic AK ratios.  With 1e6 oracle histories the ratios sit
# 0.1-0.3 % below the reference's committed means (100 kVp HVL 0.4995 against 0.5010, 30 kVp
# 0.4988 against 0.4995), with either mu_en table; the committed series quote a run-to-run
# spread below the binomial floor of their photon count, so their own error bars cannot
# carry the comparison, and the allowance stands for the difference of the two builds'
# cross-section tables.
POLY_SYSTEMATIC = 0.005


def hvl_source(golden, case):
    sc = golden["scene"]["source"]
    src = dict(position=sc["position"], direction=("disc", sc["disc_center"], sc["disc_normal"], sc["disc_radius"]))
    if case.endswith("keV"):
        src["energy"] = float(case.replace("keV", "")) * 1e3
    else:
        sp = np.array(golden["spectra"][golden["spectrum_of_case"][case]])
        src["spectrum"] = (sp[:, 0] * 1e3, sp[:, 1])
    return src


def hvl_geometry(golden, case, kind):
    if kind == "0":
        return np.full((1, 1, 1), scenes.AIR, np.uint8), (4, 4, 1e-4)
    s = golden["cases"][case]["slab_" + kind]
    return np.full((s["dims"][2], 1, 1), s["material_id"], np.uint8), s["spacing_cm"]


def hvl_tally(golden, source):
    return dict(kind="disc", spectrum=D.source_bins(source), **golden["scene"]["disc_tally"])


# ---------------------------------------------------------------- mu_en/rho ---
def test_air_mu_en_matches_reference_data_set(golden):
    """mu_en/rho of air from the EPDL tables and the transport's deposition model agrees with
    the TG-195 air table of the reference's data set (0.5 keV bin midpoints) within 1.5 % from
    4.25 to 99.75 keV, and within 0.5 % on average.  (The table's 3.75 keV row lies below its
    4.25 keV row - the argon K edge at 3.2 keV averaged into the bin - and is left out.)"""
    blob = M.TableBlob([scenes.AIR], e_max=150e3)
    t = np.array(golden["air_mu_en"])
    t = t[(t[:, 0] >= 4.25) & (t[:, 0] <= 99.75)]
    ours = blob.mu_en(0, t[:, 0] * 1e3)
    rel = ours / t[:, 1] - 1
    assert np.max(np.abs(rel)) < 0.015, np.max(np.abs(rel))
    assert np.mean(np.abs(rel)) < 0.005, np.mean(np.abs(rel))


@pytest.mark.parametrize("energy", [20e3, 60e3, 120e3])
def test_mu_en_incoherent_share_matches_compton_sampler(energy):
    """(mu_en rho - mu_photo) / mu_incoh is the mean share 1 - k'/k of an incoherent scatter;
    the oracle's Compton sampler (Kahn's method with the S(x) rejection) gives the same mean."""
    blob = M.TableBlob([scenes.WATER], e_max=150e3)
    rho = blob.blob.mat[0].density
    mu_en = blob.mu_en(0, [energy])[0]
    photo = blob.eval(0, "photo", [energy])[0]
    incoh = blob.eval(0, "incoherent", [energy])[0]
    f = (mu_en * rho - photo) / incoh
    _, kp = oracle.sample(oracle.tables_like(blob), "compton", 0, energy, 200_000, seed=9)
    share = 1 - kp
    assert abs(share.mean() - f) < 4 * share.std() / math.sqrt(share.size), (share.mean(), f)


def test_mu_en_rejects_bad_arguments():
    blob = M.TableBlob([scenes.AIR], e_max=100e3)
    with pytest.raises(N.MidsxError) as e:
        blob.mu_en(0, [150e3])
    assert e.value.status == N.TABLE_RANGE
    with pytest.raises(N.MidsxError) as e:
        blob.mu_en(3, [50e3])
    assert e.value.status == N.INVALID_ARG


# ------------------------------------------------- spectra against raw vectors ---
def test_source_bins():
    assert D.source_bins(dict(energy=30e3)) == (29999.5, 1.0, 1)
    e_min, w, n = D.source_bins(dict(spectrum=(np.array(MIDPOINTS), np.ones(239))))
    assert (e_min, w, n) == (0.0, 500.0, 239)
    # uneven lines: the grid of the smallest gap covers them all, each inside its own bin
    e = np.array([10e3, 11e3, 13e3, 16e3])
    e_min, w, n = D.source_bins(dict(spectrum=(e, np.ones(4))))
    k = np.floor((e - e_min) / w).astype(int)
    assert w == 1e3 and n == 7 and len(set(k)) == 4 and k.max() < n


@pytest.mark.parametrize("case", ["30keV", "30kVp"])
def test_spectrum_derived_quantities_equal_raw_vector_algorithm(golden, case):
    """The oracle transports the half-value-layer scene and keeps both the raw primary
    IncidentEnergy / EntranceCosine vectors (the reference's form) and the spectrum binned
    from them.  Every DerivedQuantity, computed the reference's way on the raw vectors and the
    product's way on the spectrum, agrees - the mono-energetic case includes the reference's
    double count of a line that sits on the boundary of two midpoint windows."""
    blob = M.TableBlob([scenes.AIR, scenes.ALUMINIUM], e_max=150e3)
    src = hvl_source(golden, case)
    tally = hvl_tally(golden, src)
    ids, spacing = hvl_geometry(golden, case, "hvl")
    sc = golden["scene"]
    o = oracle.run(oracle.tables_like(blob), sc["domain"], spacing, sc["slab_origin"], ids, scenes.AIR, src, [tally], n=20_000, seed=4,
                   raw_spec=0, dose=False)
    raw_e, raw_c = o["raw"]
    count, cosine = o["spectrum"][0]
    area = D.tally_area(tally)
    assert area == pytest.approx(math.pi)
    # every primary crossing is in the spectrum, at its own line
    assert count[:, 0].sum() == raw_e.size == o["scalar"][0][24]
    air = blob.dense_index(scenes.AIR)
    mu = lambda e: float(blob.mu_en(air, [e])[0])  # noqa: E731
    for cos_w in (False, True):
        for e, w in ((MIDPOINTS[59], 500.0), (30e3, 0.0), (30e3, 1000.0), (20e3, 7000.0)):
            a = OD.primary_fluence(raw_e, raw_c, area, e, w, cos_w)
            b = D.primary_fluence_from_spectrum(count, cosine, tally["spectrum"], area, e, w, cos_w)
            assert b == pytest.approx(a, rel=1e-12, abs=1e-300), (cos_w, e, w)
        a = OD.primary_spectrum_air_kerma(raw_e, raw_c, area, mu, MIDPOINTS, cos_w)
        b = sum(e * D.primary_fluence_from_spectrum(count, cosine, tally["spectrum"], area, e, 500.0, cos_w) * mu(e)
                for e in MIDPOINTS)
        assert a > 0 and b == pytest.approx(a, rel=1e-12)


@pytest.mark.parametrize("case", ["30kVp", "100kVp"])
def test_oracle_polyenergetic_hvl_through_spectrum_air_kerma(golden, case):
    """The reference's committed half- and quarter-value layers of its 30 kVp and 100 kVp
    spectra (AK_hvl / AK_0 = 1/2, AK_qvl / AK_0 = 1/4), through getPrimarySpectrumAirKerma on
    the oracle's transport: within 4 sigma of this run plus POLY_SYSTEMATIC."""
    blob = M.TableBlob([scenes.AIR, scenes.ALUMINIUM], e_max=150e3)
    src = hvl_source(golden, case)
    tally = hvl_tally(golden, src)
    sc = golden["scene"]
    air = blob.dense_index(scenes.AIR)
    n = 40_000
    ak, prim = {}, {}
    for kind, seed in (("0", 21), ("hvl", 22), ("qvl", 23)):
        ids, spacing = hvl_geometry(golden, case, kind)
        o = oracle.run(oracle.tables_like(blob), sc["domain"], spacing, sc["slab_origin"], ids, scenes.AIR, src, [tally], n=n, seed=seed,
                       dose=False)
        count, cosine = o["spectrum"][0]
        mu = blob.mu_en(air, MIDPOINTS)
        ak[kind] = sum(e * D.primary_fluence_from_spectrum(count, cosine, tally["spectrum"], math.pi, e, 500.0) * m
                       for e, m in zip(MIDPOINTS, mu))
        prim[kind] = count[:, 0].sum()
    ref = golden["cases"][case]
    for kind in ("hvl", "qvl"):
        r = ak[kind] / ak["0"]
        r_ref = ref["AK_" + kind]["mean"] / ref["AK_0"]["mean"]
        pa, pb = prim[kind] / n, prim["0"] / n
        sig = r * math.sqrt((1 - pa) / (n * pa) + (1 - pb) / (n * pb))
        assert abs(r - r_ref) < 4 * sig + POLY_SYSTEMATIC * r_ref, (kind, r, r_ref, sig)


# ------------------------------------------------------------------- GPU ---
@pytest.mark.gpu
@pytest.mark.parametrize("case", ["30keV", "100kVp"])
def test_gpu_spectrum_equals_oracle_fp64(golden, case):
    """FP64 transport on the same Philox streams as the oracle: the device spectrum (counts
    and cosine sums per line and class) equals the oracle's for all but a handful of
    histories, and the primary air kerma agrees to the same degree."""
    tables = M.Tables([scenes.AIR, scenes.ALUMINIUM], e_max=150e3)
    src_d = hvl_source(golden, case)
    tally = hvl_tally(golden, src_d)
    ids, spacing = hvl_geometry(golden, case, "hvl")
    sc = golden["scene"]
    n = 100_000
    ph = M.Phantom(tables, sc["domain"], spacing, sc["slab_origin"], ids, scenes.AIR)
    tl = M.Tallies(ph, [tally], N.DOSE_OFF)
    M.run(tables, ph, M.Source(**src_d), tl, n, seed=31, precision="fp64")
    count, cosine = tl.spectrum(0)
    o = oracle.run(oracle.tables_like(tables), sc["domain"], spacing, sc["slab_origin"], ids, scenes.AIR, src_d, [tally], n=n,
                   seed=31, dose=False)
    oc, os_ = o["spectrum"][0]
    assert oc.sum() > 0.3 * n
    assert np.abs(count - oc).sum() <= max(4, 1e-4 * oc.sum()), np.abs(count - oc).sum()
    assert np.allclose(cosine, os_, rtol=1e-4, atol=2.0)
    a = D.primary_spectrum_air_kerma(tl, 0, tables, MIDPOINTS)
    air = tables.host.dense_index(scenes.AIR)
    mu = tables.host.mu_en(air, MIDPOINTS)
    b = sum(e * D.primary_fluence_from_spectrum(oc, os_, tally["spectrum"], math.pi, e, 500.0) * m
            for e, m in zip(MIDPOINTS, mu))
    assert a == pytest.approx(b, rel=1e-3)


@pytest.mark.gpu
@pytest.mark.parametrize("precision", ["fp64", "mixed"])
@pytest.mark.parametrize("case", ["30kVp", "100kVp"])
def test_gpu_polyenergetic_hvl_through_spectrum_air_kerma(golden, case, precision):
    tables = M.Tables([scenes.AIR, scenes.ALUMINIUM], e_max=150e3)
    src_d = hvl_source(golden, case)
    tally = hvl_tally(golden, src_d)
    sc = golden["scene"]
    n = 2_000_000
    ak, prim = {}, {}
    for kind, seed in (("0", 41), ("hvl", 42), ("qvl", 43)):
        ids, spacing = hvl_geometry(golden, case, kind)
        ph = M.Phantom(tables, sc["domain"], spacing, sc["slab_origin"], ids, scenes.AIR)
        tl = M.Tallies(ph, [tally], N.DOSE_OFF)
        M.run(tables, ph, M.Source(**src_d), tl, n, seed=seed, precision=precision)
        ak[kind] = D.primary_spectrum_air_kerma(tl, 0, tables, MIDPOINTS)
        prim[kind] = tl.spectrum(0)[0][:, 0].sum()
        # the spectrum holds every primary crossing that the scalar tally counts
        assert prim[kind] == tl.scalar(0)[24]
    ref = golden["cases"][case]
    for kind in ("hvl", "qvl"):
        r = ak[kind] / ak["0"]
        r_ref = ref["AK_" + kind]["mean"] / ref["AK_0"]["mean"]
        pa, pb = prim[kind] / n, prim["0"] / n
        sig = r * math.sqrt((1 - pa) / (n * pa) + (1 - pb) / (n * pb))
        assert abs(r - r_ref) < 4 * sig + POLY_SYSTEMATIC * r_ref, (kind, r, r_ref, sig)


@pytest.mark.gpu
def test_gpu_hvl_air_kerma_with_background_fast_tracking(golden):
    """The half-value-layer scene is a thin slab in 100 cm of air: background fast tracking
    takes the air gap in a few flights instead of a few hundred Woodcock steps, and the
    spectrum air kerma agrees with the reference tracking."""
    tables = M.Tables([scenes.AIR, scenes.ALUMINIUM], e_max=150e3)
    src_d = hvl_source(golden, "30kVp")
    tally = hvl_tally(golden, src_d)
    sc = golden["scene"]
    ids, spacing = hvl_geometry(golden, "30kVp", "hvl")
    ph = M.Phantom(tables, sc["domain"], spacing, sc["slab_origin"], ids, scenes.AIR)
    n = 1_000_000
    ak, prim, steps = {}, {}, {}
    for tracking, seed in (("reference", 51), ("background_fast", 52)):
        tl = M.Tallies(ph, [tally], N.DOSE_OFF)
        M.run(tables, ph, M.Source(**src_d), tl, n, seed=seed, precision="mixed", tracking=tracking)
        ak[tracking] = D.primary_spectrum_air_kerma(tl, 0, tables, MIDPOINTS)
        prim[tracking] = tl.spectrum(0)[0][:, 0].sum()
        steps[tracking] = tl.stats()["steps"] / n
    assert steps["background_fast"] * 20 < steps["reference"], steps
    p = prim["reference"] / n
    sig = ak["reference"] * np.sqrt(2 * (1 - p) / (n * p))
    assert abs(ak["background_fast"] - ak["reference"]) < 4 * sig, (ak, sig)


@pytest.mark.gpu
def test_gpu_spectrum_mixed_matches_fp64_and_validation():
    """Mixed and FP64 forms on identical streams give the same primary spectrum (primary
    energies are exact source lines in both), and invalid spectrum specs are refused."""
    sc = scenes.water_cube(n_histories=1, n=20, bins=4)
    tables, ph, src, _ = sc.build()
    spec = dict(kind="rect", corner=(5, 5, 15), edge1=(10, 0, 0), edge2=(0, 10, 0), spectrum=(0.0, 1000.0, 70))
    out = {}
    for p in ("fp64", "mixed"):
        tl = M.Tallies(ph, [spec], N.DOSE_OFF)
        M.run(tables, ph, src, tl, 200_000, seed=3, precision=p)
        out[p] = tl.spectrum(0)
    # a primary is at 60 keV (bin 60); scattered photons spread below
    assert out["fp64"][0][60, 0] > 0 and out["fp64"][0][:60, 3].sum() > 0
    # a history whose FP32 arithmetic takes another branch is rare: the spectra agree to 0.1 %
    assert np.abs(out["fp64"][0][:, 0] - out["mixed"][0][:, 0]).sum() <= 1e-3 * out["fp64"][0][:, 0].sum() + 5
    assert np.abs(out["fp64"][0] - out["mixed"][0]).sum() <= 1e-3 * out["fp64"][0].sum() + 5
    np.testing.assert_allclose(out["mixed"][1], out["fp64"][1], rtol=1e-3, atol=1.0)
    bad = [dict(spec, spectrum=(0.0, 0.0, 10)), dict(spec, spectrum=(0.0, 1.0, -1)),
           dict(spec, spectrum=(0.0, 1.0, N.MAX_ENERGY_BINS + 1)),
           dict(kind="binned", corner=(5, 5, 15), edge1=(10, 0, 0), edge2=(0, 10, 0), nu=2, nv=2,
                spectrum=(0.0, 1.0, 4)),
           dict(kind="cuboid", min=(0, 0, 0), max=(1, 1, 1), spectrum=(0.0, 1.0, 4))]
    for b in bad:
        with pytest.raises(N.MidsxError) as e:
            M.Tallies(ph, [b], N.DOSE_OFF)
        assert e.value.status == N.INVALID_ARG
    tl = M.Tallies(ph, [dict(spec, spectrum=None)], N.DOSE_OFF)
    with pytest.raises(N.MidsxError):
        N.check(N.load().midsx_gpu_fetch_spectrum(tl.handle, 0, None, None, None), "fetch")
    # single runs score spectra with either scheduler (same trajectories: identical integer
    # words in the mixed form) and any tracking
    got = {}
    for sched in ("pool", "lanes"):
        tl = M.Tallies(ph, [spec], N.DOSE_OFF)
        M.run(tables, ph, src, tl, 50_000, seed=4, precision="mixed", scheduler=sched)
        got[sched] = tl.spectrum(0)
    np.testing.assert_array_equal(got["pool"][0], got["lanes"][0])
    np.testing.assert_array_equal(got["pool"][1], got["lanes"][1])
    for tracking in ("background_fast", "macro_cell"):
        tl = M.Tallies(ph, [spec], N.DOSE_OFF)
        M.run(tables, ph, src, tl, 1000, seed=1, tracking=tracking)
        assert tl.spectrum(0)[0].sum() > 0
    with pytest.raises(N.MidsxError) as e:
        M.run(tables, ph, src, M.Tallies(ph, [spec], N.DOSE_OFF), 100, seed=1, scheduler="lanes",
              tracking="background_fast")
    assert e.value.status == N.INVALID_ARG
