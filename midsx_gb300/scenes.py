"""Seeded synthetic workloads of the benchmark configurations.

Every input is generated from numpy.random.default_rng(seed); nothing is read from disk
except the package's own data files.  Units: cm, eV.

  water_cube      20 cm air box, 10 cm water cube at 1 mm (100^3), 60 keV pencil beam,
                  dose + 100x100 binned exit-plane tally.
  cone_beam_dose  256x256x128 voxels at 0.5 mm, 40 seeded ellipsoids of soft tissue /
                  adipose / cortical bone in air, 80 kVp Kramers spectrum filtered by
                  2.5 mm Al, point source 50 cm in front of the phantom, 20 degree cone.
  radiography     512x512x256 at 0.5 mm, same generator plus sixteen 2 mm lead spheres,
                  100 kVp, 512x512 detector of 1 mm bins at 100 cm SID.
"""
import numpy as np

from . import api
from .native import DOSE_FULL, DOSE_SUM

AIR = 3               # "Air, Dry (near sea level)"
WATER = 48            # "Water, Liquid"
SOFT_TISSUE = 153     # "Soft tissue - C5"
ADIPOSE = 170         # "Breast Adipose"
CORTICAL_BONE = 169   # "Cortical Bone - C5"
ALUMINIUM = 61        # "Al"
LEAD = 130            # "Pb"


class Scene:
    """A transport problem: materials, geometry, source and tallies."""

    def __init__(self, name, materials, domain, spacing, origin, ids, background, source, specs,
                 dose_mode, n_histories, e_max):
        self.name = name
        self.materials = materials
        self.domain = domain
        self.spacing = spacing
        self.origin = origin
        self.ids = ids
        self.background = background
        self.source = source          # dict(position, direction, energy | spectrum)
        self.specs = specs
        self.dose_mode = dose_mode
        self.n_histories = n_histories
        self.e_max = e_max

    def oracle_kwargs(self):
        return dict(domain=self.domain, spacing=self.spacing, origin=self.origin, ids=self.ids,
                    background_id=self.background, source=self.source, specs=self.specs)

    def build(self, tables=None):
        """Device objects (tables, phantom, source, tallies) for this scene."""
        t = tables or api.Tables(self.materials, e_max=self.e_max)
        ph = api.Phantom(t, self.domain, self.spacing, self.origin, self.ids, self.background)
        src = api.Source(**self.source)
        tl = api.Tallies(ph, self.specs, self.dose_mode)
        return t, ph, src, tl


def water_cube(n_histories=1_000_000, n=100, bins=100):
    """60 keV pencil beam into a 10 cm water cube voxelised at 10/n cm inside 20 cm of air."""
    ids = np.full((n, n, n), WATER, dtype=np.uint8)
    h = 10.0 / n
    specs = [dict(kind="binned", corner=(5, 5, 15), edge1=(10, 0, 0), edge2=(0, 10, 0), nu=bins, nv=bins)]
    return Scene("water_cube_60keV_pencil", [AIR, WATER], (20, 20, 20), (h, h, h), (5, 5, 5), ids, AIR,
                 dict(position=(10, 10, 0), direction=("beam", (10, 10, 20)), energy=60e3), specs,
                 DOSE_FULL, n_histories, 100e3)


def ellipsoid_phantom(shape, spacing, seed, n_ellipsoids=40, lead_spheres=0):
    """uint8 MIDSX ids shaped (nz, ny, nx): air, then ellipsoids painted in order
    (centre uniform in the inner 80% of the extent, semi-axes U(0.5, 4) cm, uniform random
    rotation, material soft tissue 0.5 / adipose 0.3 / cortical bone 0.2), then optional
    1 mm-radius lead spheres."""
    rng = np.random.default_rng(seed)
    nz, ny, nx = shape
    ext = np.array([nx, ny, nz], dtype=np.float64) * spacing
    ids = np.full(shape, AIR, dtype=np.uint8)
    zc = (np.arange(nz) + 0.5) * spacing
    yc = (np.arange(ny) + 0.5) * spacing
    xc = (np.arange(nx) + 0.5) * spacing
    mats = np.array([SOFT_TISSUE, ADIPOSE, CORTICAL_BONE])
    for _ in range(n_ellipsoids):
        c = ext * (0.1 + 0.8 * rng.random(3))
        semi = rng.uniform(0.5, 4.0, 3)
        q = rng.normal(size=4)
        q /= np.linalg.norm(q)
        w, x, y, z = q
        R = np.array([[1 - 2 * (y * y + z * z), 2 * (x * y - z * w), 2 * (x * z + y * w)],
                      [2 * (x * y + z * w), 1 - 2 * (x * x + z * z), 2 * (y * z - x * w)],
                      [2 * (x * z - y * w), 2 * (y * z + x * w), 1 - 2 * (x * x + y * y)]])
        m = mats[rng.choice(3, p=[0.5, 0.3, 0.2])]
        r = semi.max()
        lo = np.maximum(((c - r) / spacing).astype(int), 0)
        hi = np.minimum(((c + r) / spacing).astype(int) + 1, [nx, ny, nz])
        if np.any(hi <= lo):
            continue
        Z, Y, X = np.meshgrid(zc[lo[2]:hi[2]], yc[lo[1]:hi[1]], xc[lo[0]:hi[0]], indexing="ij")
        d = np.stack([X - c[0], Y - c[1], Z - c[2]], axis=-1) @ R  # body frame coordinates
        inside = ((d / semi) ** 2).sum(axis=-1) <= 1.0
        ids[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]][inside] = m
    for _ in range(lead_spheres):
        c = ext * (0.1 + 0.8 * rng.random(3))
        r = 0.1
        lo = np.maximum(((c - r) / spacing).astype(int), 0)
        hi = np.minimum(((c + r) / spacing).astype(int) + 1, [nx, ny, nz])
        Z, Y, X = np.meshgrid(zc[lo[2]:hi[2]], yc[lo[1]:hi[1]], xc[lo[0]:hi[0]], indexing="ij")
        inside = (X - c[0]) ** 2 + (Y - c[1]) ** 2 + (Z - c[2]) ** 2 <= r * r
        ids[lo[2]:hi[2], lo[1]:hi[1], lo[0]:hi[0]][inside] = LEAD
    return ids


def kramers_spectrum(kvp, e_min=10.0, al_mm=2.5, tables=None):
    """Kramers' law N(E) ~ (E0 - E) / E on 1 keV bins e_min..kvp (keV), filtered by al_mm of
    aluminium with the rebuilt Al attenuation table (`tables`: any table set whose material 0
    is aluminium, with .eval; default: built here).  Returns (energies eV, weights)."""
    e_kev = np.arange(e_min, kvp + 0.5, 1.0)
    w = (kvp - e_kev) / e_kev
    blob = tables or api.TableBlob([ALUMINIUM], e_max=max(150e3, kvp * 1e3))
    mu = blob.eval(0, "total", e_kev * 1e3)
    w = w * np.exp(-mu * al_mm / 10.0)
    return e_kev * 1e3, w


def cone_beam_dose(n_histories=100_000_000, shape=(128, 256, 256), spacing=0.05, seed=1, source_distance=50.0,
                   half_angle_deg=10.0, kvp=80.0, al=None):
    """al: tables holding aluminium first, for the filtration (default: built here)."""
    nz, ny, nx = shape
    ids = ellipsoid_phantom(shape, spacing, seed)
    ext = np.array([nx, ny, nz]) * spacing
    z0 = source_distance + 0.5
    origin = (0.0, 0.0, z0)
    domain = (ext[0], ext[1], z0 + ext[2] + 1.0)
    src_pos = (ext[0] / 2, ext[1] / 2, 0.5)
    radius = source_distance * np.tan(np.radians(half_angle_deg))
    spectrum = kramers_spectrum(kvp, tables=al)
    source = dict(position=src_pos, direction=("disc", (ext[0] / 2, ext[1] / 2, z0), (0, 0, 1), radius),
                  spectrum=spectrum)
    return Scene("cone_beam_dose_%dx%dx%d_%gkVp" % (nx, ny, nz, kvp),
                 [AIR, SOFT_TISSUE, ADIPOSE, CORTICAL_BONE], domain, (spacing,) * 3, origin, ids, AIR, source, [],
                 DOSE_FULL, n_histories, 150e3)


def batch_jobs(n_jobs=64, seed=1, edge_range=(32, 256), kvp_range=(20.0, 120.0), hist_range=(1e5, 1e8),
               hist_scale=1.0, spacing=0.1):
    """The batched configuration: n_jobs independent simulations, phantom edge log-uniform in
    edge_range voxels at `spacing` cm (seeded ellipsoid phantoms), Kramers spectra with kVp
    uniform in kvp_range, history counts log-uniform in hist_range (times hist_scale), each
    with its own per-voxel dose tally.  Returns a list of Scene."""
    rng = np.random.default_rng(seed)
    out = []
    al = api.TableBlob([ALUMINIUM], e_max=150e3)
    for j in range(n_jobs):
        edge = int(round(np.exp(rng.uniform(np.log(edge_range[0]), np.log(edge_range[1])))))
        kvp = float(np.round(rng.uniform(*kvp_range)))
        n = int(np.exp(rng.uniform(np.log(hist_range[0]), np.log(hist_range[1]))) * hist_scale)
        shape = (edge, edge, edge)
        ids = ellipsoid_phantom(shape, spacing, seed=1000 + j, n_ellipsoids=max(4, edge // 8))
        ext = edge * spacing
        z0 = 10.0 + 0.5
        domain = (ext, ext, z0 + ext + 1.0)
        spectrum = kramers_spectrum(kvp, e_min=min(10.0, kvp - 5.0), tables=al)
        source = dict(position=(ext / 2, ext / 2, 0.5), direction=("disc", (ext / 2, ext / 2, z0), (0, 0, 1), ext / 2),
                      spectrum=spectrum)
        out.append(Scene("batch_job_%d_%d^3_%gkVp" % (j, edge, kvp), [AIR, SOFT_TISSUE, ADIPOSE, CORTICAL_BONE],
                         domain, (spacing,) * 3, (0.0, 0.0, z0), ids, AIR, source, [], DOSE_FULL, max(n, 1), 150e3))
    return out


def radiography(n_histories=1_000_000_000, shape=(256, 512, 512), spacing=0.05, seed=1, det_bins=512,
                det_pitch=0.1, sid=100.0, kvp=100.0, lead_spheres=16, al=None):
    """Projection radiograph: phantom midway between a point source and a det_bins^2
    detector of det_pitch cm bins at `sid` cm (primary and scattered fluence per bin).  With
    lead_spheres=0 the tables hold the four tissue materials only (no lead majorant)."""
    nz, ny, nx = shape
    ids = ellipsoid_phantom(shape, spacing, seed, lead_spheres=lead_spheres)
    ext = np.array([nx, ny, nz]) * spacing
    det = det_bins * det_pitch
    width = max(det, ext[0])
    origin = ((width - ext[0]) / 2, (width - ext[1]) / 2, sid / 2 - ext[2] / 2)
    domain = (width, width, sid)
    src_pos = (width / 2, width / 2, 0.0)
    corner = ((width - det) / 2, (width - det) / 2, sid)
    specs = [dict(kind="binned", corner=corner, edge1=(det, 0, 0), edge2=(0, det, 0), nu=det_bins, nv=det_bins)]
    source = dict(position=src_pos, direction=("disc", (width / 2, width / 2, sid), (0, 0, 1), det / 2),
                  spectrum=kramers_spectrum(kvp, tables=al))
    materials = [AIR, SOFT_TISSUE, ADIPOSE, CORTICAL_BONE] + ([LEAD] if lead_spheres else [])
    return Scene("radiography_%dx%dx%d_%gkVp" % (nx, ny, nz, kvp), materials, domain, (spacing,) * 3, origin, ids,
                 AIR, source, specs, DOSE_SUM, n_histories, 150e3)


def dose_job(edge, spacing=0.1, seed=1, kvp=80.0, n_histories=1_000_000, al=None):
    """A dose request: edge^3 seeded ellipsoid phantom at `spacing` cm, Kramers spectrum at
    kvp, disc-collimated point source 10 cm in front of the phantom, per-voxel dose tally."""
    shape = (edge, edge, edge)
    ids = ellipsoid_phantom(shape, spacing, seed=seed, n_ellipsoids=max(4, edge // 8))
    ext = edge * spacing
    z0 = 10.5
    spectrum = kramers_spectrum(kvp, e_min=min(10.0, kvp - 5.0), tables=al)
    source = dict(position=(ext / 2, ext / 2, 0.5), direction=("disc", (ext / 2, ext / 2, z0), (0, 0, 1), ext / 2),
                  spectrum=spectrum)
    return Scene("dose_%d^3_%gkVp" % (edge, kvp), [AIR, SOFT_TISSUE, ADIPOSE, CORTICAL_BONE],
                 (ext, ext, z0 + ext + 1.0), (spacing,) * 3, (0.0, 0.0, z0), ids, AIR, source, [], DOSE_FULL,
                 n_histories, 150e3)


SERVING_CLASSES = (
    # name, probability, histories
    ("small_dose_64^3", 0.70, 1_000_000),
    ("medium_dose_128^3", 0.25, 10_000_000),
    ("radiography_256x256x128", 0.05, 100_000_000),
)


def serving_templates(pool=4, seed=1, small_edge=64, medium_edge=128, radio_shape=(128, 256, 256), radio_bins=256,
                      radio_lead=0):
    """Phantom/source/tally templates of the serving mix: `pool` seeded phantoms per class.
    Dose classes: small_edge^3 and medium_edge^3 at 1 mm with a full dose tally; radiography:
    radio_shape at 0.5 mm (radio_lead lead spheres) with a radio_bins^2 detector of 2 mm bins
    at 100 cm SID and no dose tally.  Returns {class name: [Scene]}."""
    al = api.TableBlob([ALUMINIUM], e_max=150e3)
    kvps = (60.0, 80.0, 100.0, 120.0)
    out = {}
    for ci, (name, _, n) in enumerate(SERVING_CLASSES):
        scenes = []
        for k in range(pool):
            s = seed * 1000 + ci * 100 + k
            if ci < 2:
                edge = small_edge if ci == 0 else medium_edge
                scenes.append(dose_job(edge, 0.1, s, kvps[k % len(kvps)], n, al))
            else:
                sc = radiography(n, shape=radio_shape, spacing=0.05, seed=s, det_bins=radio_bins,
                                 det_pitch=0.2, kvp=100.0, lead_spheres=radio_lead)
                sc.dose_mode = 0
                scenes.append(sc)
        out[name] = scenes
    return out


def serving_requests(rate=200.0, n_requests=400, seed=1, pool=4, hist_scale=1.0):
    """A seeded Poisson stream of requests over the classes of SERVING_CLASSES: arrival time
    (s), class name, template index, history count (times hist_scale), seed and first id."""
    rng = np.random.default_rng(seed)
    t = np.cumsum(rng.exponential(1.0 / rate, size=n_requests))
    names = [c[0] for c in SERVING_CLASSES]
    probs = np.array([c[1] for c in SERVING_CLASSES])
    cls = rng.choice(len(names), size=n_requests, p=probs / probs.sum())
    tmpl = rng.integers(0, pool, size=n_requests)
    out = []
    for i in range(n_requests):
        n = max(1, int(SERVING_CLASSES[cls[i]][2] * hist_scale))
        out.append(dict(t=float(t[i]), cls=names[cls[i]], template=int(tmpl[i]), n=n, seed=seed * 100000 + i,
                        first=0))
    return out
