"""Builders for the networks this package ships solvers for.

* ``primordial``: the 9-species + energy primordial network
  (reactions k01-k19, k21-k23 of ``primordial_rates``; every cooling action
  of ``primordial_cooling`` except ``compton``), tables of 1024 log-spaced
  bins over 1-1e9 K.
* ``primordial_compton``: the same with Compton cooling off the CMB
  (``primordial_cooling.py``'s ``compton`` action: ``-comp (1+z)^4
  (T - 2.73 (1+z)) de``), whose term reads the call's redshift and the
  cell's temperature directly; 45 tables.
* ``oxygen``: H, He and O ion-by-ion (16 equations); see :mod:`ion_by_ion`.
* ``oxygen_uvb``: the same ions under a UV background: photoionisation and
  photoheating tabulated in redshift (100 bins over z in [0, 15]).
"""

from . import reaction_classes as rc
from .chemical_network import ChemicalNetwork


PRIMORDIAL_COOLING = ("brem", "ceHI", "ceHeI", "ceHeII", "ciHI", "ciHeI", "ciHeII",
                      "ciHeIS", "gammah", "gloverabel08", "h2formation", "reHII",
                      "reHeII1", "reHeII2", "reHeIII")
PRIMORDIAL_REACTIONS = ("k01", "k02", "k03", "k04", "k05", "k06", "k07", "k08",
                        "k09", "k10", "k11", "k12", "k13", "k14", "k15", "k16",
                        "k17", "k18", "k19", "k21", "k22", "k23")


def primordial_network(T_bounds=(1.0, 1e9), n_bins=1024, with_compton=False):
    from .primordial_rates import setup_primordial
    setup_primordial()
    from . import primordial_cooling  # noqa: F401  (registers the actions)
    # The actions cache their sympy equation; a fresh setup re-creates the
    # species, so drop any cached equation built against older objects.
    for c in rc.cooling_registry.values():
        c._eq = None
    net = ChemicalNetwork()
    cooling = list(PRIMORDIAL_COOLING) + (["compton"] if with_compton else [])
    for name in cooling:
        net.add_cooling(name)
    for name in PRIMORDIAL_REACTIONS:
        net.add_reaction(name)
    net.init_temperature(T_bounds, n_bins=n_bins)
    return net


SHIPPED_NETWORKS = ("primordial", "primordial_compton", "oxygen", "oxygen_uvb")


def build_network(name):
    """The network a shipped solver is generated from, by solver name."""
    if name == "primordial":
        return primordial_network()
    if name == "primordial_compton":
        return primordial_network(with_compton=True)
    if name == "oxygen":
        from .ion_by_ion import oxygen_network
        return oxygen_network()
    if name == "oxygen_uvb":
        from .ion_by_ion import oxygen_uvb_network
        return oxygen_uvb_network()
    raise KeyError("unknown network %r" % name)
