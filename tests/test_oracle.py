"""CPU checks of the oracle and of the host table builder (no GPU).

Pins of the oracle:
* Philox4x32-10 known-answer vectors of Salmon et al. (Random123 distribution);
* the reference's own committed half-value-layer results
  (cpp_simulations/half_value_layer/data/*.txt, via tests/golden/hvl_reference.json);
* exact energy balance (source = deposited + escaped) on every run;
* the two RNG modes (per-history Philox, per-thread mt19937 as in the reference) agree
  statistically.
Table-builder checks restate the reference's table arithmetic in numpy from the raw
element data (epdl_photon.bin), independently of the C++ builder; the oracle's own table
build (oracle/tables.py) is compared with the product's array by array, and the oracle runs
on its own tables throughout.
"""
import math
import os
import struct

import numpy as np
import pytest

import midsx_gb300 as M
import oracle
from midsx_gb300 import scenes

# ------------------------------------------------------------------ Philox KATs ---
KAT = [
    ([0, 0, 0, 0], [0, 0], [0x6627e8d5, 0xe169c58d, 0xbc57ac4c, 0x9b00dbd8]),
    ([0xffffffff] * 4, [0xffffffff] * 2, [0x408f276d, 0x41c83b0e, 0xa20bc7c6, 0x6d5451fd]),
    ([0x243f6a88, 0x85a308d3, 0x13198a2e, 0x03707344], [0xa4093822, 0x299f31d0],
     [0xd16cfe09, 0x94fdcceb, 0x5001e420, 0x24126ea1]),
]


@pytest.mark.parametrize("ctr,key,expect", KAT)
def test_philox_known_answers(ctr, key, expect):
    assert oracle.philox(ctr, key) == expect


# ------------------------------------------------------------ stream layout ---
def _philox_py(ctr, key):
    """Philox4x32-10 (Salmon et al., SC'11) in plain Python, independent of the oracle."""
    x = list(ctr)
    k0, k1 = key
    M = 0xFFFFFFFF
    for r in range(10):
        if r:
            k0, k1 = (k0 + 0x9E3779B9) & M, (k1 + 0xBB67AE85) & M
        p0, p1 = 0xD2511F53 * x[0], 0xCD9E8D57 * x[2]
        x = [(p1 >> 32) ^ x[1] ^ k0, p1 & M, (p0 >> 32) ^ x[3] ^ k1, p0 & M]
    return x


def _u(word):
    return (((word << 32) >> 11) + 1) * 2.0 ** -53


def test_generator_follows_the_documented_draw_layout():
    """The history stream the device and the oracle share: event draw n is word (n & 3) of
    block (n >> 2, h_lo, h_hi, 0), each interaction starting a new block; the Woodcock-step
    pair of step index i is words (2 (i & 1), 2 (i & 1) + 1) of block (i >> 1, h_lo, h_hi,
    1 + n), i = steps so far + the parity they had at the flight segment's start."""
    seed, h = 0x0123456789ABCDEF, 0x0000000A00000007
    key = (seed & 0xFFFFFFFF, seed >> 32)
    hl, hh = h & 0xFFFFFFFF, h >> 32
    D, E, S, G = oracle.GEN_DRAW, oracle.GEN_EVENT, oracle.GEN_STEP, oracle.GEN_SEGMENT
    # a history: 3 source draws, 3 steps, an interaction (5 draws), a segment, 2 steps,
    # an interaction (2 draws), a segment, 1 step
    ops = [D, D, D] + [S, D, D] * 3 + [E] + [D] * 5 + [G] + [S, D, D] * 2 + [E, D, D, G] + [S, D, D]
    got = oracle.generator_script(seed, h, ops)
    want, n, steps, par = [], 0, 0, 0

    def event():
        nonlocal n
        w = _philox_py([n >> 2, hl, hh, 0], key)[n & 3]
        n += 1
        return _u(w)

    def step():
        nonlocal steps
        i = steps + par
        b = _philox_py([i >> 1, hl, hh, 1 + n], key)
        steps += 1
        o = 2 * (i & 1)
        return [_u(b[o]), _u(b[o + 1])]

    want += [event() for _ in range(3)]
    for _ in range(3):
        want += step()
    n = (n + 3) & ~3
    want += [event() for _ in range(5)]
    par = steps & 1
    for _ in range(2):
        want += step()
    n = (n + 3) & ~3
    want += [event() for _ in range(2)]
    par = steps & 1
    want += step()
    assert len(got) == len(want)
    np.testing.assert_array_equal(got, np.array(want))


# ----------------------------------------------------------- HVL golden results ---
def hvl_primary(blob, golden, case, kind, n, seed, rng=oracle.RNG_PHILOX):
    sc = golden["scene"]
    if kind == "0":
        ids = np.full((1, 1, 1), scenes.AIR, np.uint8)
        spacing = (4, 4, 1e-4)
    else:
        s = golden["cases"][case]["slab_" + kind]
        ids = np.full((s["dims"][2], 1, 1), s["material_id"], np.uint8)
        spacing = s["spacing_cm"]
    src = dict(position=sc["source"]["position"],
               direction=("disc", sc["source"]["disc_center"], sc["source"]["disc_normal"], sc["source"]["disc_radius"]),
               energy=float(case.replace("keV", "")) * 1e3)
    r = oracle.run(blob, sc["domain"], spacing, sc["slab_origin"], ids, scenes.AIR, src,
                   [dict(kind="disc", **sc["disc_tally"])], n=n, seed=seed, rng=rng, dose=False)
    s = r["stats"]
    assert s["deposited_grid"] + s["deposited_background"] + s["escaped_energy"] == pytest.approx(
        s["source_energy"], rel=1e-9)
    return r["scalar"][0][0]  # primary-class incident-energy count on the disc


def ratio_sigma(n_a, n_b, n):
    pa, pb = n_a / n, n_b / n
    return (n_a / n_b) * math.sqrt((1 - pa) / (n * pa) + (1 - pb) / (n * pb))


@pytest.mark.parametrize("case", ["30keV", "100keV"])
def test_oracle_reproduces_reference_hvl(golden, case):
    """Primary air-kerma ratios AK_hvl/AK_0 and AK_qvl/AK_0 of the reference's own runs
    (mono-energetic: the ratio of primary photon counts on the disc)."""
    blob = oracle.tables.tables((scenes.AIR, scenes.ALUMINIUM), 150e3)
    n = 200_000
    n0 = hvl_primary(blob, golden, case, "0", n, 11)
    ref = golden["cases"][case]
    for kind, seed in (("hvl", 12), ("qvl", 13)):
        nk = hvl_primary(blob, golden, case, kind, n, seed)
        r = nk / n0
        r_ref = ref["AK_" + kind]["mean"] / ref["AK_0"]["mean"]
        sig = math.hypot(ratio_sigma(nk, n0, n), r_ref * 1e-4)
        assert abs(r - r_ref) < 4 * sig, (kind, r, r_ref, sig)


def test_rng_modes_agree_statistically():
    sc = scenes.water_cube(n=20, bins=10)
    blob = oracle.tables_for(sc)
    a = oracle.run(blob, n=100_000, seed=3, rng=oracle.RNG_PHILOX, **sc.oracle_kwargs())["stats"]
    b = oracle.run(blob, n=100_000, seed=3, rng=oracle.RNG_MT19937, **sc.oracle_kwargs())["stats"]
    for k in ("photo", "coherent", "incoherent"):
        assert abs(a[k] - b[k]) < 5 * math.sqrt(a[k] + b[k]), k
    da, db = a["deposited_grid"], b["deposited_grid"]
    assert abs(da - db) / da < 0.01


def test_split_history_ranges_equal_one_run():
    sc = scenes.water_cube(n=10, bins=10)
    blob = oracle.tables_for(sc)
    one = oracle.run(blob, n=4000, seed=5, history=True, **sc.oracle_kwargs())
    lo = oracle.run(blob, n=2000, seed=5, first=0, history=True, **sc.oracle_kwargs())
    hi = oracle.run(blob, n=2000, seed=5, first=2000, history=True, **sc.oracle_kwargs())
    np.testing.assert_array_equal(one["history_deposit"],
                                  np.concatenate([lo["history_deposit"], hi["history_deposit"]]))


# ------------------------------------------------------------ table builder checks ---
def read_epdl(path):
    with open(path, "rb") as f:
        b = f.read()
    assert b[:8] == b"MIDSXEPD"
    _, n = struct.unpack_from("<II", b, 8)
    off = 16
    out = {}
    for _ in range(n):
        z, awr = struct.unpack_from("<Id", b, off)
        off += 12
        tabs = []
        for _ in range(5):
            (m,) = struct.unpack_from("<I", b, off)
            off += 4
            x = np.frombuffer(b, np.float64, m, off)
            off += 8 * m
            y = np.frombuffer(b, np.float64, m, off)
            off += 8 * m
            tabs.append((x, y))
        out[z] = tabs
    return out


def loglog(x, y, q):
    """LogLogLinear of the reference (interpolators.cpp:37-76) in numpy."""
    lx, ly, lq = np.log10(x), np.log10(y), np.log10(q)
    out = np.empty_like(q)
    lo = lq <= lx[0]
    hi = lq >= lx[-1]
    mid = ~(lo | hi)
    idx = np.searchsorted(lx, lq[mid], side="right")
    slope = (ly[idx] - ly[idx - 1]) / (lx[idx] - lx[idx - 1])
    out[mid] = 10 ** (ly[idx - 1] + slope * (lq[mid] - lx[idx - 1]))
    out[lo] = 10 ** ly[0]
    out[hi] = 10 ** ly[-1]
    return out


def test_single_element_photo_table_matches_raw_epdl():
    """Pure Al (id 61): photoionisation macroscopic cross section at every EPDL node equals
    N_A rho / A * sigma * 1e-24 (material_properties.cpp:66-73, material_data.cpp:56-60)."""
    data = read_epdl(os.path.join(M.DATA_DIR, "epdl_photon.bin"))
    x, y = data[13][2]
    blob = M.TableBlob([scenes.ALUMINIUM], e_max=150e3)
    n_al = 6.022140857e23 * 2.699 / 26.981538
    xs = np.unique(x)
    expect = n_al * loglog(x, y, xs) * 1e-24
    got = blob.eval(0, "photo", xs)
    np.testing.assert_allclose(got, expect, rtol=1e-12)


def test_mixture_sfunc_is_weight_fraction_average():
    """Water S(x): sum of weight fraction x element S(x) on the merged grid
    (material_data.cpp:87-114, non-macroscopic branch)."""
    data = read_epdl(os.path.join(M.DATA_DIR, "epdl_photon.bin"))
    blob = M.TableBlob([scenes.WATER], e_max=150e3)
    w = {1: 0.111898, 8: 0.888102}
    grid = np.unique(np.concatenate([data[z][4][0] for z in w]))
    q = grid[1:]  # x = 0 is a clamp node
    expect = sum(w[z] * loglog(data[z][4][0], data[z][4][1], q) for z in w)
    np.testing.assert_allclose(blob.eval(0, "sfunc", q), expect, rtol=1e-11)


def test_total_is_sum_of_components_and_majorant_dominates():
    mats = [scenes.AIR, scenes.SOFT_TISSUE, scenes.CORTICAL_BONE, scenes.LEAD]
    blob = M.TableBlob(mats, e_max=150e3)
    e = np.geomspace(1e3, 1.5e5, 2000)
    for m in range(len(mats)):
        tot = blob.eval(m, "total", e)
        parts = blob.eval(m, "coherent", e) + blob.eval(m, "incoherent", e) + blob.eval(m, "photo", e)
        np.testing.assert_allclose(tot, parts, rtol=0.02)  # log-log interpolation between nodes
        assert np.all(blob.eval(0, "majorant", e) >= tot * (1 - 1e-9))


TABLE_MATERIALS = [scenes.AIR, scenes.WATER, scenes.SOFT_TISSUE, scenes.ADIPOSE, scenes.CORTICAL_BONE,
                   scenes.ALUMINIUM, scenes.LEAD]


def test_product_tables_equal_the_oracles_independent_build():
    """The product's C++ table build (midsx_gb300/csrc/tables.cpp) against the oracle's own
    numpy restatement of the reference's construction (oracle/tables.py), array by array:
    every node grid and RITA energy grid bit-identical, log10 values within 1e-12, spline
    control points within 1e-9 (two different solvers of the collocation system), RITA rows
    of equal length with y within 1e-13 and the interpolation parameters a, b within 1e-8
    (they come from a difference of nearly equal slopes); evaluated values within 1e-10."""
    p = M.TableBlob(TABLE_MATERIALS, e_max=150e3)
    o = oracle.tables.OracleTables(TABLE_MATERIALS, 150e3)

    def lin(tp, to):
        assert tp.n == to.n
        np.testing.assert_array_equal(p.array(tp.x, tp.n), o.array(to.x, to.n))
        for f in ("lx", "ly"):
            a, b = p.array(getattr(tp, f), tp.n), o.array(getattr(to, f), to.n)
            fin = np.isfinite(a)
            np.testing.assert_array_equal(fin, np.isfinite(b))
            np.testing.assert_allclose(b[fin], a[fin], rtol=0, atol=1e-12)

    lin(p.blob.majorant, o.blob.majorant)
    rng = np.random.default_rng(7)
    e = np.exp(rng.uniform(np.log(1e3), np.log(1.5e5), 2000))
    np.testing.assert_allclose(o.eval(0, "majorant", e), p.eval(0, "majorant", e), rtol=1e-10)
    for m in range(len(TABLE_MATERIALS)):
        tp, to = p.blob.mat[m], o.blob.mat[m]
        assert tp.id == to.id and tp.density == to.density
        for name in ("total", "photo", "sfunc", "ffactor"):
            lin(getattr(tp, name), getattr(to, name))
        for name in ("coh", "incoh"):
            sp, so = getattr(tp, name), getattr(to, name)
            assert (sp.n_ctrl, sp.degree) == (so.n_ctrl, so.degree)
            assert sp.lx_min == so.lx_min and sp.lx_max == so.lx_max
            nk = sp.n_ctrl + sp.degree + 1
            np.testing.assert_allclose(o.array(so.knot_u, nk), p.array(sp.knot_u, nk), rtol=0, atol=1e-15)
            np.testing.assert_allclose(o.array(so.ctrl, so.n_ctrl), p.array(sp.ctrl, sp.n_ctrl), rtol=0, atol=1e-9)
        for which in ("total", "photo", "coherent", "incoherent"):
            np.testing.assert_allclose(o.eval(m, which, e), p.eval(m, which, e), rtol=1e-10, err_msg=which)
        rp, ro = tp.rita, to.rita
        assert (rp.n_energy, rp.n_rows) == (ro.n_energy, ro.n_rows)
        np.testing.assert_array_equal(p.array(rp.energy, rp.n_energy), o.array(ro.energy, ro.n_energy))
        np.testing.assert_array_equal(p.iarray(rp.row_start, rp.n_energy + 1), o.iarray(ro.row_start, ro.n_energy + 1))
        np.testing.assert_array_equal(p.array(rp.x, rp.n_rows), o.array(ro.x, ro.n_rows))
        for f, tol in (("y", 1e-13), ("a", 1e-8), ("b", 1e-8)):
            a, b = p.array(getattr(rp, f), rp.n_rows), o.array(getattr(ro, f), ro.n_rows)
            fin = np.isfinite(a)
            np.testing.assert_array_equal(fin, np.isfinite(b))
            np.testing.assert_allclose(b[fin], a[fin], rtol=tol, atol=tol, err_msg=f)


def test_spline_collocation_solved_from_raw_epdl_nodes():
    """Water's coherent LogLogSpline rebuilt from the raw EPDL nodes without either builder:
    the element tables of H and O (epdl_photon.bin) through the element splines (scipy's
    make_interp_spline with the averaged knots, a banded solver of its own), weighted by the
    number densities on the merged grid, and the material spline solved again by scipy.  The
    product's table gives the same values at the nodes and between them."""
    from scipy.interpolate import make_interp_spline
    data = read_epdl(os.path.join(M.DATA_DIR, "epdl_photon.bin"))
    blob = M.TableBlob([scenes.WATER], e_max=150e3)

    def loglog_spline(x, y):
        lx, ly = np.log10(x), np.log10(y)
        lo, hi = lx.min(), lx.max()
        u = (lx - lo) / (hi - lo)
        p = min(x.size - 1, 3)
        t = np.zeros(x.size + p + 1)
        for j in range(1, x.size - p):
            t[j + p] = u[j:j + p].mean()
        t[x.size:] = 1.0
        b = make_interp_spline(u, ly, k=p, t=t)
        return lambda q: 10 ** b((np.log10(q) - lo) / (hi - lo))

    w = {1: 0.111898, 8: 0.888102}
    awt = {1: 1.00794, 8: 15.9994}
    grid = np.unique(np.concatenate([data[z][0][0] for z in w]))
    y = sum(6.022140857e23 * 1.0 * w[z] / awt[z] * loglog_spline(*data[z][0])(grid) for z in w) * 1e-24
    coh = loglog_spline(grid, y)
    np.testing.assert_allclose(blob.eval(0, "coherent", grid), y, rtol=1e-9)
    q = np.sqrt(grid[1:] * grid[:-1])
    q = q[(q > 1e3) & (q < 1.5e5)]
    np.testing.assert_allclose(blob.eval(0, "coherent", q), coh(q), rtol=1e-9)


ALPHA = 0.51099895000E6 / (math.sqrt(2.0) * 4.135667662e-15 * 299792458E2 * 1E8)


def rayleigh_pdf(blob, m, mu, energy):
    """(1 + mu^2) F(x)^2 with x = alpha k sqrt(1 - mu) (material_data.cpp:62-73)."""
    x = ALPHA * energy / 0.51099895000E6 * np.sqrt(1 - mu)
    f = blob.eval(m, "ffactor", x)
    return (1 + mu * mu) * f * f


def test_rita_rows_are_monotone_cdfs():
    """RITA rows are CDFs over [-1, 1].  The reference normalises the PDF with a 1001-point
    Simpson rule (probability_dist.cpp:267-287) but integrates the CDF adaptively, so for a
    forward-peaked PDF the last CDF value is (true integral) / (Simpson estimate) < 1; the
    test predicts that value with an independent fine integration."""
    blob = M.TableBlob([scenes.WATER, scenes.LEAD], e_max=150e3)
    for m in range(2):
        r = blob.blob.mat[m].rita
        E = blob.array(r.energy, r.n_energy)
        rows = blob.iarray(r.row_start, r.n_energy + 1)
        X = blob.array(r.x, r.n_rows)
        Y = blob.array(r.y, r.n_rows)
        for k in range(r.n_energy):
            if E[k] < 1e3:
                continue  # below ~400 eV the reference's form-factor lookup yields NaN rows
            x = X[rows[k]:rows[k + 1]]
            y = Y[rows[k]:rows[k + 1]]
            assert x[0] == -1 and x[-1] == 1
            assert np.all(np.diff(x) > 0) and np.all(np.diff(y) >= 0)
            if k % 8 == 0 or E[k] > 5e4:
                h = 2.0 / 1000
                mu = -1 + h * np.arange(1001)
                mu[-1] = 1.0
                w = np.where(np.arange(1001) % 2 == 1, 4.0, 2.0)
                w[0] = w[-1] = 1.0
                simpson = h / 3 * np.sum(w * rayleigh_pdf(blob, m, mu, E[k]))
                t = np.linspace(0, 1, 400001)  # fine grid in s = sqrt(1 - mu), dense at mu = 1
                mus = 1 - 2 * t * t
                g = rayleigh_pdf(blob, m, mus, E[k])
                # between x = 0 and the first form-factor node the reference's LogLogLinear
                # is NaN; the integrand there is ~(1 + mu^2) F(0)^2
                g = np.where(np.isnan(g), rayleigh_pdf(blob, m, np.ones(1), E[k])[0], g) * 4 * t
                true = np.sum((g[1:] + g[:-1]) / 2 * np.diff(t))
                assert abs(y[-1] - true / simpson) < 2e-4, (m, E[k], y[-1], true / simpson)


def test_scenes_are_deterministic():
    a = scenes.ellipsoid_phantom((16, 32, 32), 0.2, seed=4)
    b = scenes.ellipsoid_phantom((16, 32, 32), 0.2, seed=4)
    np.testing.assert_array_equal(a, b)
    e, w = scenes.kramers_spectrum(80.0)
    assert e.size == 71 and w[-1] == 0 and np.all(w[:-1] > 0)


def test_serving_stream_is_seeded_poisson_with_the_class_mix():
    a = scenes.serving_requests(rate=200.0, n_requests=4000, seed=1)
    b = scenes.serving_requests(rate=200.0, n_requests=4000, seed=1)
    assert a == b
    t = np.array([r["t"] for r in a])
    gaps = np.diff(np.concatenate([[0.0], t]))
    assert np.all(gaps > 0) and abs(gaps.mean() - 1 / 200.0) < 0.1 / 200.0
    frac = {c: np.mean([r["cls"] == c for r in a]) for c, _, _ in scenes.SERVING_CLASSES}
    for c, p, n in scenes.SERVING_CLASSES:
        assert abs(frac[c] - p) < 0.03, (c, frac[c])
        assert all(r["n"] == n for r in a if r["cls"] == c)
    assert len({r["seed"] for r in a}) == len(a)


def test_serving_templates_shapes_and_tables():
    tm = scenes.serving_templates(pool=2, seed=3, small_edge=16, medium_edge=24, radio_shape=(16, 32, 32),
                                  radio_bins=32)
    assert [sc.ids.shape for sc in tm["small_dose_64^3"]] == [(16, 16, 16)] * 2
    radio = tm["radiography_256x256x128"][0]
    assert radio.dose_mode == 0 and radio.specs[0]["nu"] == 32 and scenes.LEAD not in radio.materials
    lead = scenes.serving_templates(pool=1, seed=3, small_edge=8, medium_edge=8, radio_shape=(16, 32, 32),
                                    radio_bins=8, radio_lead=2)["radiography_256x256x128"][0]
    assert scenes.LEAD in lead.materials and (lead.ids == scenes.LEAD).any()
