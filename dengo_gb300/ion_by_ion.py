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
seed derived from the ion's name.  The same tables feed the GPU solver and the
oracle.  Photo-ionisation/heating (HM12 tables) are not set up.
"""

import hashlib

import numpy as np

from .periodic_table import periodic_table_by_name
from .reaction_classes import (AtomicSpecies, CoolingAction, Reaction, registry_setup,
                               species_registry)

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


@registry_setup
def setup_ionization(atom_name, photo_background=None, cooling=True):
    """Register the ions of ``atom_name`` with their ionisation,
    recombination and cooling terms; returns the new names."""
    if photo_background is not None:
        raise NotImplementedError("photo-ionisation tables (HM12) are not available here")
    num = periodic_table_by_name[atom_name][0]
    de = species_registry["de"]
    ions = {i: AtomicSpecies(atom_name, i) for i in range(num + 1)}
    for i in range(num + 1):
        s = ions[i]
        sm1, sp1 = ions.get(i - 1), ions.get(i + 1)
        if sp1 is not None:
            Reaction("%s_i" % s.name, ionization_rate(atom_name, i),
                     [(1, s), (1, de)], [(1, sp1), (2, de)])
        if sm1 is not None:
            Reaction("%s_r" % s.name, recombination_rate(atom_name, i),
                     [(1, s), (1, de)], [(1, sm1)])
        if cooling:
            act = CoolingAction("%s_c" % s.name, "-%s_c * %s * de" % (s.name, s.name))
            act.tables["%s_c" % s.name] = cooling_rate(atom_name, i)


def oxygen_network(T_bounds=(1e0, 1e10), n_bins=8192):
    """H, He and O ion by ion with electrons and energy: 16 equations,
    22 reactions, 14 cooling tables, 8192 log-T bins."""
    from .chemical_network import ChemicalNetwork
    net = ChemicalNetwork()
    net.add_species("de")
    for atom in ("H", "O", "He"):
        s, c, r = setup_ionization(atom)
        net.add_collection(s, c, r)
    net.init_temperature(T_bounds, n_bins=n_bins)
    return net
