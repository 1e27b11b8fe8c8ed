"""Network-definition model: species, reactions, cooling actions, registries.

This mirrors the reference's public model (dengo/reaction_classes.py:43-377)
so that network scripts written for the reference run unchanged:

* ``species_registry`` / ``reaction_registry`` / ``cooling_registry`` are
  module-level dicts filled as objects are created
  (reference: reaction_classes.py:43-45).
* ``Species`` / ``ChemicalSpecies`` / ``AtomicSpecies`` / ``MolecularSpecies``
  name and weight species exactly as the reference does
  (reaction_classes.py:273-320), because the names fix the state-vector order
  (species are sorted by ``"Species: <name>"``) and the weights are emitted as
  literals into the generated code.
* ``Reaction`` builds ``net_change * k * prod(reactants)`` as a sympy
  expression (reaction_classes.py:86-165); ``CoolingAction`` evaluates its
  equation string against the species and table symbols and substitutes its
  temporaries (reaction_classes.py:322-375).

The sympy trees built here must be identical to the reference's, since the C
and CUDA code is printed from them and floating-point evaluation order follows
the printed order.  Two details matter for that:

* Rate coefficients are instances of a ``sympy.Symbol`` subclass named
  ``ReactionCoefficient``; sympy orders factors by class name, which puts the
  rate first in every product (``k08[i]*H_1*H_m0``).
* A rate's derivative by the energy term is zero.  In the reference the
  derivative hook compares a sympy symbol with a ``Species`` object
  (chemical_network.py:83, reaction_classes.py:77-84) and never fires, so the
  generated Jacobian's ``ge`` column is identically zero.  The same holds here.
"""

import functools

import sympy

from .periodic_table import periodic_table_by_name
from .exceptions import UnknownCoolingAction, UnknownReaction, UnknownSpecies

species_registry = {}
reaction_registry = {}
cooling_registry = {}

_REGISTRIES = (species_registry, cooling_registry, reaction_registry)


def registry_setup(func):
    """Decorate a network-setup function so it returns what it registered.

    The wrapped call returns ``[new_species, new_cooling, new_reactions]``,
    three sets of names (reference: reaction_classes.py:47-59), which
    ``ChemicalNetwork.add_collection`` accepts directly.
    """

    @functools.wraps(func)
    def wrapper(*args, **kwargs):
        before = [set(reg) for reg in _REGISTRIES]
        func(*args, **kwargs)
        return [set(reg) - old for reg, old in zip(_REGISTRIES, before)]

    return wrapper


def ensure_reaction(r):
    if isinstance(r, Reaction):
        return r
    if r not in reaction_registry:
        raise UnknownReaction(r)
    return reaction_registry[r]


def ensure_cooling(c):
    if isinstance(c, CoolingAction):
        return c
    if c not in cooling_registry:
        raise UnknownCoolingAction(c)
    return cooling_registry[c]


def ensure_species(s):
    if isinstance(s, Species):
        return s
    if s not in species_registry:
        raise UnknownSpecies(s)
    return species_registry[s]


count_m = sympy.Symbol("m", integer=True)
index_i = sympy.Idx("i", count_m)


@functools.total_ordering
class ComparableMixin:
    """Total order and hash through ``_cmpkey`` (reference: dengo/mixin.py:5-34)."""

    def _cmpkey(self):
        raise NotImplementedError

    def __eq__(self, other):
        try:
            return self._cmpkey() == other._cmpkey()
        except AttributeError:
            return NotImplemented

    def __lt__(self, other):
        try:
            return self._cmpkey() < other._cmpkey()
        except AttributeError:
            return NotImplemented

    def __hash__(self):
        return hash(self._cmpkey())


class ReactionCoefficient(sympy.Symbol):
    """Symbol standing for one interpolated rate, printed as ``<name>[i]``.

    ``energy`` is set by ``ChemicalNetwork.add_reaction`` for interface
    compatibility.  Differentiation treats the coefficient as a constant: the
    generated Jacobian has no rate-temperature terms, as in the reference.
    """

    energy = None


class Species(ComparableMixin):
    """A state variable of the network (reference: reaction_classes.py:273-285)."""

    def __init__(self, name, weight, pretty_name=None):
        self.name = name
        self.weight = weight
        self.pretty_name = pretty_name or name
        self.symbol = sympy.Symbol(name)
        species_registry[name] = self

    def _cmpkey(self):
        return repr(self)

    def __repr__(self):
        return "Species: %s" % self.name


class ChemicalSpecies(Species):
    """A species with a charge state (reference: reaction_classes.py:287-297)."""

    def __init__(self, name, weight, free_electrons=0.0, pretty_name=None):
        self.free_electrons = free_electrons
        super().__init__(name, weight, pretty_name)

    def number_density(self, quantities):
        q = quantities[self.name]
        return q if self.weight == 0 else q / self.weight


class AtomicSpecies(ChemicalSpecies):
    """An ion of an element: ``H_1`` is neutral H, ``H_2`` is H+, ``H_m0`` is H-.

    Naming follows reaction_classes.py:299-310.
    """

    def __init__(self, atom_name, free_electrons):
        _, weight, element = periodic_table_by_name[atom_name]
        if free_electrons < 0:
            name = "%s_m%i" % (atom_name, abs(free_electrons + 1))
        else:
            name = "%s_%01i" % (atom_name, free_electrons + 1)
        self.atom_name = atom_name
        super().__init__(name, weight, free_electrons,
                         "%s with %s free electrons" % (element, free_electrons))


class MolecularSpecies(ChemicalSpecies):
    """A molecule or molecular ion, named ``<molecule>_<free_electrons+1>``
    (reaction_classes.py:312-320)."""

    def __init__(self, molecule_name, weight, free_electrons, original_name=None):
        name = "%s_%i" % (molecule_name, free_electrons + 1)
        self.original_name = original_name or molecule_name
        super().__init__(name, weight, free_electrons,
                         "%s with %s free electrons" % (name, free_electrons))


class Reaction(ComparableMixin):
    """A mass-action reaction ``sum(n_l * L) -> sum(n_r * R)`` with rate table.

    ``coeff_fn(network)`` returns the rate on ``network.T`` (or ``network.z``
    for photo-rates whose name contains ``pi``).  The symbolic contribution to
    species ``s`` is ``net_change(s) * k * prod(L**n_l)``
    (reaction_classes.py:148-165).
    """

    def __init__(self, name, coeff_fn, left_side, right_side):
        self.name = name
        self.coeff_fn = coeff_fn
        self.coeff_sym = ReactionCoefficient("%s[i]" % name)
        self.left_side = left_side
        self.right_side = right_side
        self.considered = {s.name for _, s in left_side + right_side}
        reaction_registry[name] = self

    def __contains__(self, c):
        return ensure_species(c).name in self.considered

    @property
    def down_species(self):
        return [s for _, s in self.left_side]

    @property
    def up_species(self):
        return [s for _, s in self.right_side]

    @property
    def species(self):
        return set(self.down_species + self.up_species)

    def net_change(self, sname):
        gained = sum(n for n, s in self.right_side if s.name == sname)
        lost = sum(n for n, s in self.left_side if s.name == sname)
        return gained - lost

    def __call__(self, quantities, up_derivatives, down_derivatives):
        r = self.rate(quantities)
        for n, s in self.left_side:
            r *= s.number_density(quantities) ** n
        for n, s in self.left_side:
            down_derivatives[s.name] += r * n * s.weight
        for n, s in self.right_side:
            up_derivatives[s.name] += r * n * s.weight
        return r

    def _cmpkey(self):
        return repr(self)

    def __repr__(self):
        lhs = " + ".join("%s*%s" % (n, s.name) for n, s in self.left_side)
        rhs = " + ".join("%s*%s" % (n, s.name) for n, s in self.right_side)
        return "%s : %s => %s" % (self.name, lhs, rhs)

    @classmethod
    def create_reaction(cls, name, left_side, right_side):
        def register(f):
            cls(name, f, left_side, right_side)
        return register

    @property
    def lhs_equation(self):
        eq = self.coeff_sym
        for n, s in self.left_side:
            for _ in range(n):
                eq = eq * s.symbol
        return eq

    def species_equation(self, species):
        if isinstance(species, str):
            species = species_registry[species]
        elif isinstance(species, (sympy.IndexedBase, sympy.Symbol)):
            species = species_registry[str(species)]
        if species not in self.species:
            return 0
        return self.net_change(species.name) * self.lhs_equation


reaction = Reaction.create_reaction


class CoolingAction:
    """A heating/cooling term of the energy equation.

    ``equation`` is a Python expression over species names, the action's
    table names and its temporaries.  Tables become symbols
    ``<action>_<table>[i]``; temporaries are expanded in place
    (reaction_classes.py:333-351).  Temporaries are parsed with the species
    and table symbols in scope, so a temporary that names a species (e.g. the
    ``galdl`` density sum of ``gloverabel08``) depends on that species.
    """

    def __init__(self, name, equation):
        self.name = name
        self._equation = equation
        self._eq = None
        self.tables = {}
        self.temporaries = {}
        self.table_symbols = {}
        self.temp_symbols = {}
        cooling_registry[name] = self

    def __lt__(self, other):
        return self.name < other.name

    def _species_symbols(self):
        return {n: s.symbol for n, s in species_registry.items()}

    @property
    def equation(self):
        if self._eq is not None:
            return self._eq
        tables = {n: sympy.Symbol("%s_%s[i]" % (self.name, n)) for n in self.tables}
        temps = {n: sympy.Symbol(n) for n in self.temporaries}
        self.table_symbols.update(tables)
        self.temp_symbols.update(temps)
        namespace = self._species_symbols()
        namespace.update(tables)
        namespace.update(temps)
        eq = eval(compile(self._equation, "<cooling %s>" % self.name, "eval"),
                  {"__builtins__": {}}, namespace)
        scope = self._species_symbols()
        scope.update(tables)
        for tname, texpr in self.temporaries.items():
            eq = eq.subs(tname, sympy.sympify(texpr, locals=scope))
        self._eq = eq
        return eq

    @property
    def species(self):
        eq = self.equation
        skip = set(self.temp_symbols.values()) | set(self.table_symbols.values())
        return {species_registry[str(s).replace("[i]", "")]
                for s in eq.atoms(sympy.Symbol) if s not in skip}

    def table(self, func):
        self.tables[func.__name__] = func

    def temporary(self, name, eq):
        self.temporaries[name] = eq

    @classmethod
    def create_cooling_action(cls, name, equation):
        obj = cls(name, equation)

        def apply(f):
            f(obj)
        return apply


cooling_action = CoolingAction.create_cooling_action


# -- ion-by-ion registration helpers (reaction_classes.py:167-198, 200-271,
# 379-441, 443-514 of the reference).  Each registers the same reactions and
# cooling actions, under the same names and conditions, as the reference's
# function of that name and returns the new names.  The reference tabulates
# them from CHIANTI, Gnat & Ferland's cooling tables and the HM12 UV
# background; those data are not available, so the tables come from the
# seeded synthetic curves of :mod:`dengo_gb300.ion_by_ion`.

def _ion_stage(species):
    """(element, stage) of an AtomicSpecies named ``<El>_<stage + 1>``."""
    ion_name = species.name.lower()
    if "_" not in ion_name:
        raise RuntimeError("Name must be in 'Ion Species' format: %s" % species.name)
    element, state = ion_name.split("_")[:2]
    return element, int(state) - 1


def chianti_rate(atom_name, sm1, s, sp1):
    """Collisional ionisation ``<s>_i`` (s + e -> sp1 + 2e, when ``sp1``
    exists) and recombination ``<s>_r`` (s + e -> sm1, when ``sm1``
    exists)."""
    from .ion_by_ion import ionization_rate, recombination_rate
    _, stage = _ion_stage(s)
    de = species_registry["de"]
    new_rates = []
    if sp1 is not None:
        Reaction("%s_i" % s.name, ionization_rate(atom_name, stage),
                 [(1, s), (1, de)], [(1, sp1), (2, de)])
        new_rates.append("%s_i" % s.name)
    if sm1 is not None:
        Reaction("%s_r" % s.name, recombination_rate(atom_name, stage),
                 [(1, s), (1, de)], [(1, sm1)])
        new_rates.append("%s_r" % s.name)
    return new_rates


def ion_cooling_rate(species, atom_name):
    """Cooling action ``<s>_c``: ``-<s>_c * <s> * de`` with one table."""
    from .ion_by_ion import cooling_rate
    _, stage = _ion_stage(species)
    act = CoolingAction("%s_c" % species.name, "-%s_c * %s * de" % (species.name, species.name))
    act.tables["%s_c" % species.name] = cooling_rate(atom_name, stage)
    return ["%s_c" % species.name]


def ion_photoionization_rate(species, photo_background="HM12"):
    """Photoionisation ``<s>_pi`` (s -> next ion + e), tabulated in
    redshift, when the next ion is registered."""
    from .ion_by_ion import photo_rate
    element, stage = _ion_stage(species)
    nxt = "%s_%s" % (element.capitalize(), stage + 2)
    if nxt not in species_registry:
        return []
    Reaction("%s_pi" % species.name, photo_rate(element, species.name.lower(), "photoionization"),
             [(1, species)], [(1, species_registry[nxt]), (1, species_registry["de"])])
    return ["%s_pi" % species.name]


def ion_photoheating_rate(species, photo_background="HM12"):
    """Photoheating cooling action ``<s>_ph``: ``<s>_ph * <s>``, tabulated in
    redshift."""
    from .ion_by_ion import photo_rate
    element, _ = _ion_stage(species)
    if species.name not in species_registry:
        return []
    act = CoolingAction("%s_ph" % species.name, "%s_ph * %s" % (species.name, species.name))
    act.tables["%s_ph" % species.name] = photo_rate(element, species.name.lower(), "photoheating")
    return ["%s_ph" % species.name]
