"""Interaction tables of the CPU oracle, built independently of the product - TEST
INFRASTRUCTURE ONLY.

The product builds its tables in C++ (midsx_gb300/csrc/tables.cpp).  The oracle must not
share them: a table-construction error would then sit on both sides of every parity test.
This module restates the reference's table construction from the published methods, in
numpy, reading only the element data files (epdl_photon.bin, elements.txt, materials.txt):

  MaterialProperties::setNumberDensity      src/MIDSX/Core/material_properties.cpp:66-73
  MaterialData::calculateWeightedAverageOfColumns (merged energy grid, weight fraction or
      number-density weights, per-element LogLogLinear / LogLogSpline)
                                            src/MIDSX/Core/material_data.cpp:87-114
  MaterialData total cross section on the merged grid of the three interaction tables
                                            src/MIDSX/Core/material_data.cpp:24-27,75-85,125-134
  InteractionData majorant (per-node maximum of the materials' totals on their merged grid)
                                            src/MIDSX/Core/interaction_data.cpp:42-73
  Interpolator::LogLogLinear / LogLogSpline src/MIDSX/Core/interpolators.cpp:3-76
  ContinuousInversion (RITA) construction   src/MIDSX/Core/probability_dist.cpp:121-287
  mergeMatrices (sort + unique)             include/MIDSX/Core/material_helpers.h:69-85

The LogLogSpline is Eigen's SplineFitting::Interpolate (a third-party dependency absent from
the reference checkout): global B-spline interpolation through the points with parameters
u = scaled log10 x, degree min(n - 1, 3), knots by averaging (Piegl & Tiller, "The NURBS
Book", eq. 9.8) and the collocation system solved densely (here by LAPACK's LU through
numpy; the product uses a banded elimination, Eigen a full-pivot LU).  Values therefore agree
with the product's to about 1e-12 relative, not bit for bit.

The blob this module fills has the layout of midsx_table_blob (include/midsx_gpu.h), so the
oracle's C++ loop reads it as it would read the product's; RITA rows are built for the
incoherent-grid energies up to the first node >= e_max, as the product does (the reference
builds them for the whole grid; rows above the source energy are never used).
"""
import ctypes as C
import functools
import os
import struct

import numpy as np

from midsx_gb300 import native as N  # structure layouts only: this loads no library

DATA_DIR = os.path.join(os.path.dirname(os.path.dirname(os.path.abspath(__file__))), "midsx_gb300", "data")

# include/MIDSX/Core/constants.h:16-23
ELECTRON_REST_MASS = 0.51099895000E6
PLANCK_CONSTANT = 4.135667662e-15
SPEED_OF_LIGHT = 299792458E2
AVOGADRO_CONSTANT = 6.022140857e23
ALPHA = ELECTRON_REST_MASS / (np.sqrt(2.0) * PLANCK_CONSTANT * SPEED_OF_LIGHT * 1E8)

TABLES = ("coh", "incoh", "photo", "ffactor", "sfunc")  # order of the element records


# ------------------------------------------------------------------------ data files ---
@functools.lru_cache(maxsize=4)
def load_data(data_dir=DATA_DIR):
    """(elements {Z: {awr, coh, incoh, photo, ffactor, sfunc: (x, y)}}, atomic weights {Z: w},
    materials {id: (name, density, [(Z, weight fraction)] ascending Z)})."""
    with open(os.path.join(data_dir, "epdl_photon.bin"), "rb") as f:
        raw = f.read()
    if raw[:8] != b"MIDSXEPD":
        raise ValueError("not an epdl_photon.bin file")
    version, n = struct.unpack_from("<II", raw, 8)
    if version != 1:
        raise ValueError("unknown epdl_photon.bin version %d" % version)
    off = 16
    elements = {}
    for _ in range(n):
        z, awr = struct.unpack_from("<Id", raw, off)
        off += 12
        rec = {"awr": awr}
        for name in TABLES:
            (k,) = struct.unpack_from("<I", raw, off)
            off += 4
            x = np.frombuffer(raw, dtype="<f8", count=k, offset=off).copy()
            off += 8 * k
            y = np.frombuffer(raw, dtype="<f8", count=k, offset=off).copy()
            off += 8 * k
            rec[name] = (x, y)
        elements[z] = rec
    weights = {}
    for line in open(os.path.join(data_dir, "elements.txt")):
        if line.strip() and not line.startswith("#"):
            p = line.rstrip("\n").split("|")
            weights[int(p[0])] = float(p[2])
    materials = {}
    for line in open(os.path.join(data_dir, "materials.txt")):
        if line.strip() and not line.startswith("#"):
            p = line.rstrip("\n").split("|")
            comp = sorted((int(a), float(b)) for a, b in (c.split(":") for c in p[3].split(",")))
            materials[int(p[0])] = (p[1], float(p[2]), comp)
    return elements, weights, materials


# -------------------------------------------------------------------- interpolators ---
class LogLogLinear:
    """Interpolator::LogLogLinear: linear interpolation of log10 y in log10 x, clamped to the
    end values.  The interval is found on the raw x values (upper_bound), the monotone
    equivalent of the reference's search on log10 x."""

    def __init__(self, x, y):
        self.x = np.asarray(x, dtype=np.float64)
        with np.errstate(divide="ignore", invalid="ignore"):
            self.lx = np.log10(self.x)
            self.ly = np.log10(np.asarray(y, dtype=np.float64))

    def __call__(self, q):
        q = np.asarray(q, dtype=np.float64)
        x, lx, ly = self.x, self.lx, self.ly
        n = x.size
        idx = np.searchsorted(x, q, side="right")
        lo = q <= x[0]
        hi = q >= x[-1]
        i = np.clip(idx, 1, n - 1)
        with np.errstate(divide="ignore", invalid="ignore"):
            lq = np.log10(q)
            slope = (ly[i] - ly[i - 1]) / (lx[i] - lx[i - 1])
            v = ly[i - 1] + slope * (lq - lx[i - 1])
        v = np.where(lo, ly[0], np.where(hi, ly[-1], v))
        return np.power(10.0, v)


class LogLogSpline:
    """Interpolator::LogLogSpline: a B-spline through (u_i, log10 y_i) with u = (log10 x -
    min) / (max - min), degree min(n - 1, 3), averaged knots, evaluated as 10^spline(u)."""

    def __init__(self, x, y):
        x = np.asarray(x, dtype=np.float64)
        lx = np.log10(x)
        ly = np.log10(np.asarray(y, dtype=np.float64))
        n = x.size
        if n < 2:
            raise ValueError("a spline needs two points")
        self.lx_min, self.lx_max = float(lx.min()), float(lx.max())
        u = (lx - self.lx_min) / (self.lx_max - self.lx_min)
        p = min(n - 1, 3)
        self.degree = p
        knots = np.zeros(n + p + 1)
        for j in range(1, n - p):
            knots[j + p] = u[j:j + p].sum() / p
        knots[n:] = 1.0
        self.knots = knots
        # collocation matrix: row i holds the basis functions at u_i (end rows interpolate the
        # end points exactly), solved densely
        A = np.zeros((n, n))
        A[0, 0] = 1.0
        A[n - 1, n - 1] = 1.0
        if n > 2:
            span = self.span(u[1:-1])
            Nb = self.basis(span, u[1:-1])
            rows = np.arange(1, n - 1)
            for k in range(p + 1):
                A[rows, span - p + k] = Nb[:, k]
        self.ctrl = np.linalg.solve(A, ly)
        with np.errstate(over="ignore"):
            self.knot_e = np.power(10.0, self.lx_min + knots * (self.lx_max - self.lx_min))

    def span(self, u):
        """Knot span (NURBS Book A2.1 as Eigen's Spline::Span clamps it)."""
        p, k = self.degree, self.knots
        s = np.searchsorted(k[p - 1:k.size - p - 1], u, side="right") + (p - 1) - 1
        return np.where(u <= k[0], p, s)

    def basis(self, span, u):
        """The p + 1 non-zero basis functions at u (NURBS Book A2.2), one row per query."""
        p, k = self.degree, self.knots
        m = u.size
        Nb = np.zeros((m, p + 1))
        Nb[:, 0] = 1.0
        left = np.zeros((m, p + 1))
        right = np.zeros((m, p + 1))
        for j in range(1, p + 1):
            left[:, j] = u - k[span + 1 - j]
            right[:, j] = k[span + j] - u
            saved = np.zeros(m)
            for r in range(j):
                temp = Nb[:, r] / (right[:, r + 1] + left[:, j - r])
                Nb[:, r] = saved + right[:, r + 1] * temp
                saved = left[:, j - r] * temp
            Nb[:, j] = saved
        return Nb

    def __call__(self, e):
        e = np.atleast_1d(np.asarray(e, dtype=np.float64))
        u = (np.log10(e) - self.lx_min) / (self.lx_max - self.lx_min)
        span = self.span(u)
        Nb = self.basis(span, u)
        v = np.zeros(e.size)
        for i in range(self.degree + 1):
            v += self.ctrl[span - self.degree + i] * Nb[:, i]
        return np.power(10.0, v)


def merge(*grids):
    return np.unique(np.concatenate([np.asarray(g, dtype=np.float64) for g in grids]))


# ------------------------------------------------------------------------ materials ---
def weighted_average(elements, weights, material, table, macroscopic):
    """calculateWeightedAverageOfColumns: every element's table interpolated on the merged
    energy grid of the material's elements, summed with weight fractions (or number
    densities N_A rho w / A when macroscopic)."""
    name, density, comp = material
    gx = merge(*[elements[z][table][0] for z, _ in comp])
    gy = np.zeros(gx.size)
    for z, w in comp:
        x, y = elements[z][table]
        weight = AVOGADRO_CONSTANT * density * w / weights[z] if macroscopic else w
        interp = LogLogSpline(x, y) if table in ("coh", "incoh") else LogLogLinear(x, y)
        gy += weight * interp(gx)
    return gx, gy


class RitaBuilder:
    """ContinuousInversion's table for one energy: the Rayleigh angular PDF
    (1 + mu^2) F(x)^2 with x = ALPHA k sqrt(1 - mu), normalised by a 1001-point Simpson rule,
    a grid that starts at 10 points on [-1, 1] and halves every interval whose interpolation
    error (51-point trapezoid of |p - p_RITA|, PENELOPE eqs. 1.55-1.57) exceeds 1e-4, the CDF by
    51-point Simpson rules per interval, and the rational-interpolation parameters a, b."""

    def __init__(self, ffactor, energy, err_thresh=1e-4):
        self.ff = ffactor
        self.E = float(energy)
        self.err = err_thresh
        xs = np.linspace(-1.0, 1.0, 1001)
        w = np.where(np.arange(1001) % 2 == 1, 4.0, 2.0)
        w[0] = w[-1] = 1.0
        self.norm = (2.0 / 1000) / 3 * float(np.dot(w, self.pdf(xs)))

    def pdf(self, mu):
        k = self.E / ELECTRON_REST_MASS
        with np.errstate(invalid="ignore"):
            x = ALPHA * k * np.sqrt(1 - mu)
        f = self.ff(x)
        return (1 + mu * mu) * f * f

    def npdf(self, mu):
        return self.pdf(mu) / self.norm

    def cdf(self, xg):
        npts = 51
        h = (xg[1:] - xg[:-1]) / (npts - 1)
        pts = xg[:-1, None] + np.arange(npts)[None, :] * h[:, None]
        w = np.where(np.arange(npts) % 2 == 1, 4.0, 2.0)
        w[0] = w[-1] = 1.0
        inc = h / 3 * (self.npdf(pts) * w[None, :]).sum(axis=1)
        return np.concatenate([[0.0], np.cumsum(inc)])

    def params(self, xg, y):
        s = (y[1:] - y[:-1]) / (xg[1:] - xg[:-1])
        p0, p1 = self.npdf(xg[:-1]), self.npdf(xg[1:])
        b = 1 - s ** 2 * (1 / (p0 * p1))
        a = s * (1 / p0) - b - 1
        return a, b

    @staticmethod
    def p_rita(x, xi, xi1, yi, yi1, a, b):
        tau = (x - xi) / (xi1 - xi)
        c = 1 + a + b - a * tau
        with np.errstate(divide="ignore", invalid="ignore"):
            eta = c / (2 * b * tau) * (1 - np.sqrt(1 - 4 * b * tau * tau / c ** 2))
        eta = np.where(tau == 0, 0.0, eta)
        return (1 + a * eta + b * eta * eta) ** 2 / ((1 + a + b) * (1 - b * eta * eta)) * (yi1 - yi) / (xi1 - xi)

    def interval_errors(self, xg, y, a, b):
        nsub = 51
        xi, xi1 = xg[:-1, None], xg[1:, None]
        yi, yi1 = y[:-1, None], y[1:, None]
        A, B = a[:, None], b[:, None]
        dx = (xg[1:] - xg[:-1]) / nsub
        xk = xg[:-1, None] + np.arange(1, nsub)[None, :] * dx[:, None]
        inner = np.abs(self.npdf(xk) - self.p_rita(xk, xi, xi1, yi, yi1, A, B)).sum(axis=1)
        ends = (np.abs(self.npdf(xg[1:]) - self.p_rita(xg[1:, None], xi, xi1, yi, yi1, A, B)[:, 0]) +
                np.abs(self.npdf(xg[:-1]) - self.p_rita(xg[:-1, None], xi, xi1, yi, yi1, A, B)[:, 0]))
        return dx * (inner + ends / 2)

    def build(self):
        step = 2.0 / 9.0
        xg = np.array([-1.0 + i * step for i in range(9)] + [1.0])
        for _ in range(64):
            y = self.cdf(xg)
            a, b = self.params(xg, y)
            eps = self.interval_errors(xg, y, a, b)
            split = eps > self.err
            if not split.any():
                break
            mids = (xg[:-1] + xg[1:]) / 2
            out = []
            for i in range(xg.size - 1):
                out.append(xg[i])
                if split[i]:
                    out.append(mids[i])
            out.append(xg[-1])
            xg = np.array(out)
        else:
            raise RuntimeError("RITA refinement did not converge")
        y = self.cdf(xg)
        a, b = self.params(xg, y)
        # the last row's parameters: the reference's table has one fewer (a, b) than x; the
        # blob keeps a zero pair there
        return xg, y, np.append(a, 0.0), np.append(b, 0.0)


class MaterialTables:
    def __init__(self, mid, data, e_max):
        elements, weights, materials = data
        if mid not in materials:
            raise KeyError("unknown material id %d" % mid)
        m = materials[mid]
        self.id, self.density = mid, m[1]
        self.incoh_x, incoh_y = weighted_average(elements, weights, m, "incoh", True)
        self.coh_x, coh_y = weighted_average(elements, weights, m, "coh", True)
        self.photo_x, photo_y = weighted_average(elements, weights, m, "photo", True)
        self.incoh_y, self.coh_y, self.photo_y = incoh_y * 1E-24, coh_y * 1E-24, photo_y * 1E-24
        self.incoh = LogLogSpline(self.incoh_x, self.incoh_y)
        self.coh = LogLogSpline(self.coh_x, self.coh_y)
        self.photo = LogLogLinear(self.photo_x, self.photo_y)
        self.total_x = merge(self.incoh_x, self.coh_x, self.photo_x)
        self.total_y = self.incoh(self.total_x) + self.coh(self.total_x) + self.photo(self.total_x)
        self.total = LogLogLinear(self.total_x, self.total_y)
        self.sf_x, self.sf_y = weighted_average(elements, weights, m, "sfunc", False)
        self.ff_x, self.ff_y = weighted_average(elements, weights, m, "ffactor", False)
        self.sf = LogLogLinear(self.sf_x, self.sf_y)
        self.ff = LogLogLinear(self.ff_x, self.ff_y)
        k = int(np.searchsorted(self.incoh_x, e_max, side="left")) + 1
        if k > self.incoh_x.size or self.incoh_x[k - 1] < e_max or k < 2:
            raise ValueError("e_max beyond the incoherent energy grid")
        self.rita_e = self.incoh_x[:k].copy()
        self.rita = [RitaBuilder(self.ff, e).build() for e in self.rita_e]


# ------------------------------------------------------------------------ the blob ---
class OracleTables:
    """The oracle's own tables of a material list, as a midsx_table_blob the oracle library
    reads (.ptr), with the accessors the tests use on the product's TableBlob (.blob,
    .array, .iarray, .eval, .ids, .e_max, .dense_index)."""

    def __init__(self, material_ids, e_max=150e3, data_dir=DATA_DIR):
        data = load_data(data_dir)
        self.ids = [int(m) for m in material_ids]
        if not 1 <= len(self.ids) <= N.MAX_MATERIALS or len(set(self.ids)) != len(self.ids):
            raise ValueError("1..32 distinct material ids")
        self.e_max = float(e_max)
        self.mats = [MaterialTables(m, data, self.e_max) for m in self.ids]
        mx = merge(*[m.total_x for m in self.mats])
        my = np.max([m.total(mx) for m in self.mats], axis=0)
        self.majorant = LogLogLinear(mx, my)
        d, idata = [], []
        size = [0]

        def push(v):
            off = size[0]
            v = np.asarray(v, dtype=np.float64)
            d.append(v)
            size[0] += v.size
            return off

        def lin(t, interp):
            t.x, t.lx, t.ly, t.n = push(interp.x), push(interp.lx), push(interp.ly), interp.x.size

        def spl(t, s):
            t.knot_e, t.knot_u, t.ctrl = push(s.knot_e), push(s.knots), push(s.ctrl)
            t.n_ctrl, t.degree, t.lx_min, t.lx_max = s.ctrl.size, s.degree, s.lx_min, s.lx_max

        b = N.TableBlob()
        b.version, b.n_materials, b.e_max = 1, len(self.ids), self.e_max
        lin(b.majorant, self.majorant)
        for i, m in enumerate(self.mats):
            t = b.mat[i]
            t.id, t.density = m.id, m.density
            lin(t.total, m.total)
            lin(t.photo, m.photo)
            lin(t.sfunc, m.sf)
            lin(t.ffactor, m.ff)
            spl(t.coh, m.coh)
            spl(t.incoh, m.incoh)
            r = t.rita
            r.n_energy = m.rita_e.size
            r.energy = push(m.rita_e)
            r.log_energy = push(np.log(m.rita_e))
            r.row_start = len(idata)
            rows = 0
            for xg, _, _, _ in m.rita:
                idata.append(rows)
                rows += xg.size
            idata.append(rows)
            r.n_rows = rows
            for field, col in (("x", 0), ("y", 1), ("a", 2), ("b", 3)):
                setattr(r, field, push(np.concatenate([row[col] for row in m.rita])))
        self._data = np.ascontiguousarray(np.concatenate(d))
        self._idata = np.ascontiguousarray(np.array(idata, dtype=np.int64))
        b.n_data, b.data = self._data.size, self._data.ctypes.data_as(C.POINTER(C.c_double))
        b.n_idata, b.idata = self._idata.size, self._idata.ctypes.data_as(C.POINTER(C.c_int64))
        self._blob = b
        self.ptr = C.pointer(b)

    @property
    def blob(self):
        return self._blob

    def array(self, off, n):
        return self._data[off:off + n]

    def iarray(self, off, n):
        return self._idata[off:off + n]

    def dense_index(self, mid):
        return self.ids.index(mid)

    def eval(self, material, which, x):
        """Table values at x: 'total', 'photo', 'coherent', 'incoherent', 'sfunc', 'ffactor',
        'majorant' (material ignored)."""
        x = np.asarray(x, dtype=np.float64)
        if which == "majorant":
            return self.majorant(x)
        m = self.mats[int(material)]
        f = {"total": m.total, "photo": m.photo, "coherent": m.coh, "incoherent": m.incoh, "sfunc": m.sf,
             "ffactor": m.ff}[which]
        return f(x).reshape(x.shape)


@functools.lru_cache(maxsize=16)
def tables(material_ids, e_max=150e3):
    """Cached OracleTables of a tuple of material ids."""
    return OracleTables(material_ids, e_max)
