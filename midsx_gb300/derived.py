"""DerivedQuantity over the device's incident-energy spectra (reference:
src/MIDSX/Core/derived_quantities.cpp:3-68).

The reference scans a surface tally's raw IncidentEnergy / EntranceCosine vectors for primary
photons with energy in [energy - width/2, energy + width/2].  The GPU tallies keep an
incident-energy spectrum instead (a disc or rect tally with ``spectrum=(e_min, e_width, n)``);
a bin counts when its centre lies in the window.  A primary photon keeps its source energy, so
with bins centred on the source's lines (``source_bins``) every primary sits at a bin centre
and the sums equal the reference's.
"""
import math

import numpy as np

AIR_ID = 3  # "Air, Dry (near sea level)", derived_quantities.cpp:50


def source_bins(source):
    """(e_min, e_width, n) with one bin centred on each line of a source dict's spectrum
    (``energy=`` or ``spectrum=(energies, probabilities)``): the spacing of the grid is the
    smallest gap between lines; a single energy gets a 1 eV bin."""
    if source.get("spectrum") is None:
        e = float(source["energy"])
        return (e - 0.5, 1.0, 1)
    e = np.unique(np.asarray(source["spectrum"][0], dtype=np.float64))
    if e.size == 1:
        return (float(e[0]) - 0.5, 1.0, 1)
    step = float(np.min(np.diff(e)))
    n = int(math.floor((e[-1] - e[0]) / step + 0.5)) + 1
    return (float(e[0]) - 0.5 * step, step, n)


def tally_area(spec):
    """Area of a disc (pi r^2) or rectangle (|edge1 x edge2|) tally (surface_tally.cpp:59-88)."""
    if spec["kind"] == "disc":
        return math.pi * float(spec["radius"]) ** 2
    return float(np.linalg.norm(np.cross(np.asarray(spec["edge1"], float), np.asarray(spec["edge2"], float))))


def window_bins(spectrum, energy, width):
    """Indices of the bins whose centre lies in [energy - width/2, energy + width/2] (a relative
    1e-12 of slack keeps a zero-width window on a centre that rounds by one unit)."""
    e_min, w, n = float(spectrum[0]), float(spectrum[1]), int(spectrum[2])
    centres = e_min + (np.arange(n) + 0.5) * w
    slack = 1e-12 * max(abs(energy), abs(w))
    return np.nonzero((centres >= energy - width / 2 - slack) & (centres <= energy + width / 2 + slack))[0]


def primary_fluence_from_spectrum(count, cosine, spectrum, area, energy, width, cosine_weighted=False):
    """getPrimaryFluence over spectrum arrays shaped (n_energy, 4): primaries (class 0) per
    unit area, or the sum of their entrance cosines per unit area."""
    k = window_bins(spectrum, energy, width)
    col = cosine if cosine_weighted else count
    return float(np.asarray(col)[k, 0].sum()) / area


def primary_fluence(tallies, i, energy, width, cosine_weighted=False, stream=None):
    """DerivedQuantity::getPrimaryFluence for surface tally i of a midsx_gb300.Tallies, 1/cm^2."""
    spec = tallies.specs[i]
    if spec.get("spectrum") is None:
        raise RuntimeError("surface tally %d keeps no incident-energy spectrum" % i)
    count, cosine = tallies.spectrum(i, stream)
    return primary_fluence_from_spectrum(count, cosine, spec["spectrum"], tally_area(spec), energy, width,
                                         cosine_weighted)


def air_mu_en(tables, energy):
    """mu_en/rho (cm2/g) of material id 3 (air) in `tables` (Tables or TableBlob)."""
    blob = getattr(tables, "host", tables)
    if AIR_ID not in blob.ids:
        raise KeyError("material id %d (air) is not among the tables' materials" % AIR_ID)
    return float(blob.mu_en(blob.dense_index(AIR_ID), [energy])[0])


def primary_air_kerma(tallies, i, tables, energy, width, cosine_weighted=False, mu_en=None, stream=None):
    """DerivedQuantity::getPrimaryAirKerma: energy * fluence * mu_en/rho(air), eV/g.  mu_en, a
    callable of the energy, replaces the tables' own coefficient."""
    m = mu_en(energy) if mu_en is not None else air_mu_en(tables, energy)
    return energy * primary_fluence(tallies, i, energy, width, cosine_weighted, stream) * m


def primary_spectrum_air_kerma(tallies, i, tables, energy_spectrum, cosine_weighted=False, mu_en=None,
                               stream=None):
    """DerivedQuantity::getPrimarySpectrumAirKerma: the air kerma summed over evenly spaced
    bin midpoints, width = the spacing of the first two."""
    es = [float(e) for e in energy_spectrum]
    if len(es) < 2:
        raise ValueError("an energy spectrum needs at least two midpoints")
    width = es[1] - es[0]
    spec = tallies.specs[i]
    if spec.get("spectrum") is None:
        raise RuntimeError("surface tally %d keeps no incident-energy spectrum" % i)
    count, cosine = tallies.spectrum(i, stream)
    area = tally_area(spec)
    total = 0.0
    for e in es:
        m = mu_en(e) if mu_en is not None else air_mu_en(tables, e)
        total += e * primary_fluence_from_spectrum(count, cosine, spec["spectrum"], area, e, width,
                                                   cosine_weighted) * m
    return total
