"""DerivedQuantity restated over raw vectors - TEST INFRASTRUCTURE ONLY (the checker of
midsx_gb300.derived).

The reference's algorithm as written (src/MIDSX/Core/derived_quantities.cpp:3-68): scan the
primary IncidentEnergy vector of a surface tally, keep the values in the closed window
[energy - width/2, energy + width/2], count them (or sum the matching EntranceCosine values)
and divide by the tally's area; air kerma multiplies by energy and mu_en/rho of air; the
spectrum form sums air kerma over evenly spaced midpoints with width = their spacing.  The raw
vectors come from oracle.run(..., raw_spec=i).
"""
import numpy as np


def primary_fluence(raw_energy, raw_cosine, area, energy, width, cosine_weighted=False):
    """derived_quantities.cpp:3-45."""
    e = np.asarray(raw_energy)
    sel = (e >= energy - width / 2) & (e <= energy + width / 2)
    total = float(np.asarray(raw_cosine)[sel].sum()) if cosine_weighted else float(sel.sum())
    return total / area


def primary_air_kerma(raw_energy, raw_cosine, area, mu_en, energy, width, cosine_weighted=False):
    """derived_quantities.cpp:47-55; mu_en: callable of the energy (cm2/g)."""
    return energy * primary_fluence(raw_energy, raw_cosine, area, energy, width, cosine_weighted) * mu_en(energy)


def primary_spectrum_air_kerma(raw_energy, raw_cosine, area, mu_en, energy_spectrum, cosine_weighted=False):
    """derived_quantities.cpp:57-68."""
    es = list(energy_spectrum)
    width = es[1] - es[0]
    return sum(primary_air_kerma(raw_energy, raw_cosine, area, mu_en, e, width, cosine_weighted) for e in es)
