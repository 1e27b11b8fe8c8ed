"""Ion-by-ion networks (dengo/ion_by_ion.py:33-56).

``setup_ionization(atom)`` registers every ionisation stage of an element
(``AtomicSpecies(atom, i)``, i = 0..Z) and, as the reference does
(reaction_classes.py:168-198, 379-441):

* ``<ion>_i``: collisional ionisation  ion + e -> next ion + 2 e  (not for the
  bare nucleus);
* ``<ion>_r``: recombination  ion + e -> previous ion  (not for the neutral);
* ``<ion>_c``: a cooling action ``-<ion>_c * <ion> * de`` with one table.

The reference tabulates these from CHIANTI (ChiantiPy) and from Gnat &
Ferland's HDF5 cooling tables.  Neither is available here, so the tables are
seeded smooth synthetic curves of the physical shape (``synthetic_rates``):
ionisation ~ T^1/2 exp(-chi/kT), recombination ~ T^-0.7, cooling ~ T^1/2
exp(-chi/kT), with ionisation potentials and amplitudes drawn per ion from a
seed derived from the ion's name.  The UV-background tables (HM12) are
replaced the same way (``photo_data``), and the reference's own redshift
interpolation and extrapolation turn them into rate tables (``photo_rate``).
The same tables feed the GPU solver and the oracle.
"""

import hashlib

import numpy as np

from .periodic_table import periodic_table_by_name
from .reaction_classes import (AtomicSpecies, chianti_rate, ion_cooling_rate,
                               ion_photoheating_rate, ion_photoionization_rate, registry_setup)

_EV_K = 1.1605e4  # K per eV


def _ion_rng(name):
    seed = int.from_bytes(hashlib.sha256(name.encode()).digest()[:8], "little")
    return np.random.Generator(np.random.PCG64(seed))


def _chi_ev(atom, stage):
    """Synthetic ionisation potential of stage ``stage`` (0 = neutral)."""
    num = periodic_table_by_name[atom][0]
    rng = _ion_rng("chi:%s:%d" % (atom, stage))
    return 13.6 * (stage + 1) ** 1.6 * num ** 0.35 * rng.uniform(0.8, 1.2)


def ionization_rate(atom, stage):
    rng = _ion_rng("ion:%s:%d" % (atom, stage))
    amp = 10 ** rng.uniform(-11.0, -9.5)
    chi = _chi_ev(atom, stage) * _EV_K

    def rate(network):
        T = network.T
        return amp * np.sqrt(T) * np.exp(-np.minimum(chi / T, 700.0))
    return rate


def recombination_rate(atom, stage):
    rng = _ion_rng("rec:%s:%d" % (atom, stage))
    amp = 10 ** rng.uniform(-12.5, -11.0) * stage ** 1.5

    def rate(network):
        T = network.T
        return amp * (T / 1e4) ** -0.7 / (1.0 + (T / 1e6) ** 0.7)
    return rate


def cooling_rate(atom, stage):
    rng = _ion_rng("cool:%s:%d" % (atom, stage))
    amp = 10 ** rng.uniform(-23.5, -21.5)
    chi = _chi_ev(atom, max(stage - 1, 0)) * _EV_K * 0.5

    def rate(network):
        T = network.T
        return amp * np.sqrt(T / 1e4) * np.exp(-np.minimum(chi / T, 700.0)) + 1e-30
    return rate


def photo_data(element, ion_name, kind):
    """Seeded synthetic stand-in for the ion-by-ion UV-background tables the
    reference reads (input/photoionization/<el>_ion_by_ion_photoionization_
    <bg>.h5, input/photoheating/...; datasets ``z`` and ``<ion>``): 60
    redshifts in [0.01, 15], a log-normal bump in 1 + z per ion."""
    rng = _ion_rng("%s:%s:%s" % (kind, element, ion_name))
    z = np.logspace(-2.0, np.log10(15.0), 60)
    lo, hi = (-13.5, -11.0) if kind == "photoionization" else (-25.5, -23.0)
    amp = 10 ** rng.uniform(lo, hi)
    zp = rng.uniform(1.5, 3.5)
    vals = amp * np.exp(-0.5 * ((np.log1p(z) - np.log1p(zp)) / 0.6) ** 2) + amp * 1e-3
    return z, vals


def photo_rate(element, ion_name, kind):
    """Redshift table of a photoionisation rate or photoheating term: the
    reference's interpolation and log-space extrapolation
    (reaction_classes.py:214-260, 457-503, end_method 0), same numpy
    operations, on the tables of ``photo_data``."""
    def rate(network):
        dataz, dataS = photo_data(element, ion_name, kind)
        vals = np.interp(network.z, dataz, dataS)
        vals = np.log10(vals)
        logz = np.log10(network.z)
        logdataz = np.log10(dataz)
        logdataS = np.log10(dataS)
        extrapdown = logdataS[0] + \
            (logz - logdataz[0]) * (logdataS[0] - logdataS[1]) \
            / (logdataz[0] - logdataz[1])
        vals[logz < logdataz[0]] = extrapdown[logz < logdataz[0]]
        extrapup = logdataS[-1] + \
            (logz - logdataz[-1]) * (logdataS[-1] - logdataS[-2]) \
            / (logdataz[-1] - logdataz[-2])
        vals[logz > logdataz[-1]] = extrapup[logz > logdataz[-1]]
        vals = 10.0**vals
        return vals
    return rate


def _register_ions(atom_name, photo_background=None, cooling=True):
    """Register the ions of ``atom_name`` and their terms, in the reference's
    order (dengo/ion_by_ion.py:33-56); returns the names of everything
    registered: [species, cooling actions, reactions]."""
    num = periodic_table_by_name[atom_name][0]
    ions = {i: AtomicSpecies(atom_name, i) for i in range(num + 1)}
    names = [{s.name for s in ions.values()}, set(), set()]
    for i in range(num + 1):
        s = ions[i]
        names[2].update(chianti_rate(atom_name, ions.get(i - 1), s, ions.get(i + 1)))
        if cooling:
            names[1].update(ion_cooling_rate(s, atom_name))
        if i != num and photo_background is not None:
            names[2].update(ion_photoionization_rate(s, photo_background=photo_background))
            if cooling:
                names[1].update(ion_photoheating_rate(s, photo_background=photo_background))
    return names


@registry_setup
def setup_ionization(atom_name, photo_background=None, cooling=True):
    """Register the ions of ``atom_name`` with their ionisation,
    recombination and cooling terms; returns the new names (the reference's
    registry_setup contract).  With a ``photo_background`` every ion but the
    bare nucleus also gets ``<ion>_pi`` (photoionisation, ion -> next ion +
    e) and, with cooling, ``<ion>_ph`` (photoheating ``<ion>_ph * <ion>``),
    tabulated in redshift (reaction_classes.py:200-271, 443-514)."""
    _register_ions(atom_name, photo_background, cooling)


def oxygen_uvb_network(T_bounds=(1e0, 1e10), n_bins=8192, z_bounds=(0.0, 15.0), n_z_bins=100):
    """The oxygen network under a (synthetic) UV background: photoionisation
    and photoheating of every ion, tabulated on 100 redshifts over [0, 15]."""
    from .chemical_network import ChemicalNetwork
    net = ChemicalNetwork()
    net.add_species("de")
    for atom in ("H", "O", "He"):
        net.add_collection(*_register_ions(atom, photo_background="HM12"))
    net.init_temperature(T_bounds, n_bins=n_bins)
    net.init_redshift(z_bounds, n_z_bins=n_z_bins)
    return net


def oxygen_network(T_bounds=(1e0, 1e10), n_bins=8192):
    """H, He and O ion by ion with electrons and energy: 16 equations,
    22 reactions, 14 cooling tables, 8192 log-T bins."""
    from .chemical_network import ChemicalNetwork
    net = ChemicalNetwork()
    net.add_species("de")
    for atom in ("H", "O", "He"):
        net.add_collection(*_register_ions(atom))
    net.init_temperature(T_bounds, n_bins=n_bins)
    return net
