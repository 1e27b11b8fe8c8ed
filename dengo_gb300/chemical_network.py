"""``ChemicalNetwork``: collects species, reactions and cooling, builds the
symbolic right-hand side and Jacobian, and writes a GB300 solver.

The public surface follows the reference's class
(dengo/chemical_network.py:38-328).  The symbolic pieces (``species_total``,
``print_ccode``, ``print_jacobian_component``, ``print_mass_density``,
``temperature_calculation``) build the same sympy expressions so that the
emitted code evaluates the same floating-point operations in the same order.
``write_solver`` renders this package's CUDA template family instead of the
reference's C++ one; see :mod:`dengo_gb300.codegen`.
"""

import os

import numpy as np
import sympy

from .chemistry_constants import tevk, tiny, mh  # noqa: F401  (re-exported)
from .codegen.printers import ccode_ref
from .reaction_classes import (ChemicalSpecies, Species, cooling_registry,  # noqa: F401
                               count_m, ensure_cooling, ensure_reaction, index_i,
                               reaction_registry, species_registry)

ge = Species("ge", 1.0, "Gas Energy")
de = ChemicalSpecies("de", 1.0, pretty_name="Electrons")


class ChemicalNetwork:
    """A reaction/cooling network over a fixed, sorted set of species.

    The state vector of every generated solver is ``sorted(required_species)``
    (order by ``"Species: <name>"``), with the energy term ``ge`` included.
    """

    energy_term = None
    skip_weight = ("ge", "de")

    def __init__(self, write_intermediate=False, stop_time=3.1557e13):
        self.reactions = {}
        self.cooling_actions = {}
        self.required_species = set()
        self.write_intermediate_solutions = write_intermediate
        self.energy_term = species_registry["ge"]
        self.required_species.add(self.energy_term)
        self.stop_time = stop_time
        self.z_bounds = (0.0, 0.0)
        self.input_is_number = False

    # ---- assembling the network (chemical_network.py:54-97) -------------
    def add_collection(self, species_names, cooling_names, reaction_names):
        for s in species_names:
            self.add_species(s)
        for c in cooling_names:
            self.add_cooling(c, False)
        for r in reaction_names:
            self.add_reaction(r, False)

    def add_species(self, species):
        self.required_species.add(species_registry.get(species, species))

    def add_reaction(self, reaction, auto_add=True):
        reaction = ensure_reaction(reaction)
        if reaction.name in self.reactions:
            raise RuntimeError("reaction %s already in network" % reaction.name)
        for _, s in reaction.left_side + reaction.right_side:
            if auto_add:
                self.required_species.add(s)
            elif s not in self.required_species:
                raise RuntimeError("species %s of %s not in network"
                                   % (s.name, reaction.name))
        self.reactions[reaction.name] = reaction
        reaction.coeff_sym.energy = self.energy_term

    def add_cooling(self, cooling_term, auto_add=True):
        cooling_term = ensure_cooling(cooling_term)
        if cooling_term.name in self.cooling_actions:
            raise RuntimeError("cooling %s already in network" % cooling_term.name)
        if auto_add:
            self.required_species.update(cooling_term.species)
        else:
            missing = [s for s in cooling_term.species if s not in self.required_species]
            if missing:
                raise RuntimeError("species %s of %s not in network"
                                   % (missing, cooling_term.name))
        self.cooling_actions[cooling_term.name] = cooling_term

    # ---- grids (chemical_network.py:99-116) ----------------------------
    def init_temperature(self, T_bounds=(1, 1e8), n_bins=1024):
        self.n_bins = n_bins
        self.T = np.logspace(np.log(T_bounds[0]), np.log(T_bounds[1]),
                             n_bins, base=np.e)
        self.logT = np.log(self.T)
        self.tev = self.T / tevk
        self.logtev = np.log(self.tev)
        self.T_bounds = T_bounds

    def init_redshift(self, z_bounds=(0.0, 10.0), n_z_bins=100):
        self.n_z_bins = n_z_bins
        self.z = np.logspace(np.log(z_bounds[0] + 1.0), np.log(z_bounds[1] + 1.0),
                             n_z_bins, base=np.e)
        self.z -= 1.0
        with np.errstate(divide="ignore"):
            self.logz = np.log(self.z)
        self.z_bounds = z_bounds

    # ---- symbolic system (chemical_network.py:118-208) -----------------
    @property
    def ordered_species(self):
        """The state-vector order: ``sorted(required_species)``."""
        return sorted(self.required_species)

    def species_total(self, species):
        eq = sympy.sympify("0")
        for _, rxn in sorted(self.reactions.items()):
            eq += rxn.species_equation(species)
        return eq

    def species_reactions(self, species):
        return [rxn for _, rxn in sorted(self.reactions.items()) if species in rxn]

    def species_list(self):
        return [s.name for s in sorted(self.required_species)]

    def __iter__(self):
        for _, rxn in sorted(self.reactions.items()):
            yield rxn

    def cooling_equation(self):
        """Sum of all cooling-action equations: the raw ``d ge / dt`` numerator."""
        eq = sympy.sympify("0")
        for name in self.cooling_actions:
            eq += self.cooling_actions[name].equation
        return eq

    def rhs_expression(self, species):
        """Symbolic d(species)/dt before the ``ge`` row's division by mass density."""
        if species == self.energy_term:
            return self.cooling_equation()
        return self.species_total(species)

    def jacobian_expression(self, s1, s2):
        """d rhs(s1) / d s2, as the reference's ``print_jacobian_component``
        forms it (chemical_network.py:153-168)."""
        if s1 == self.energy_term:
            st = sum(self.cooling_actions[ca].equation
                     for ca in sorted(self.cooling_actions))
        else:
            st = self.species_total(s1)
        return sympy.diff(st, s2.symbol)

    def print_ccode(self, species, assign_to=None):
        if assign_to is None:
            assign_to = sympy.Symbol("d_%s[i]" % species.name)
        return ccode_ref(self.rhs_expression(species), assign_to=assign_to)

    def print_cooling(self, assign_to):
        return ccode_ref(self.cooling_equation(), assign_to=assign_to)

    def print_jacobian_component(self, s1, s2, assign_to=None):
        if assign_to is None:
            assign_to = sympy.Symbol("d_%s_%s" % (s1.name, s2.name))
        return ccode_ref(self.jacobian_expression(s1, s2), assign_to=assign_to)

    def mass_density_expression(self):
        eq = sympy.sympify("0")
        for s in sorted(self.required_species):
            if s.weight > 0 and s.name not in self.skip_weight:
                eq += s.symbol * s.weight
        return eq

    def print_mass_density(self):
        return ccode_ref(self.mass_density_expression())

    def species_gamma(self, species):
        # The reference tests the pre-rename names, so every species of the
        # shipped networks (including H2_1/H2_2) uses gamma = 5/3
        # (chemical_network.py:179-184).
        if species.name in ("H2I", "H2II"):
            return sympy.Symbol("gammaH2")
        return sympy.Symbol("gamma")

    def gamma_factor(self):
        eq = sympy.sympify("0")
        for s in sorted(self.required_species):
            if s.name != "ge":
                eq += sympy.sympify(s.name) / (self.species_gamma(s) - 1.0)
        return eq

    def temperature_expression(self, derivative=False):
        g = sympy.Symbol("ge")
        f = (sympy.Symbol("density") * g * sympy.Symbol("mh")) / \
            (sympy.Symbol("kb") * self.gamma_factor())
        return sympy.diff(f, g) if derivative else f

    def temperature_calculation(self, derivative=False):
        return ccode_ref(self.temperature_expression(derivative))

    # ---- initial-condition helpers (chemical_network.py:211-256) -------
    def _zeros(self, values):
        return np.zeros_like(next(iter(values.values())))

    def calculate_number_density(self, values, skip=()):
        n = self._zeros(values)
        for s in self.required_species:
            if s.name not in self.skip_weight:
                n += values[s.name] / s.weight
        return n

    def calculate_free_electrons(self, values):
        n = self._zeros(values)
        for s in self.required_species:
            if s.name not in self.skip_weight:
                n += (values[s.name] / s.weight) * s.free_electrons
        return n

    def calculate_mass_density(self, values):
        n = self._zeros(values)
        for s in self.required_species:
            if s.name not in self.skip_weight:
                n += values[s.name] * s.weight
        return n

    def calculate_total_density(self, values):
        n = self._zeros(values)
        for s in self.required_species:
            if s.name not in self.skip_weight:
                n += values[s.name]
        return n

    def convert_to_mass_density(self, values, skip=()):
        for s in self.required_species:
            if s.name not in self.skip_weight:
                values[s.name] = values[s.name] * s.weight
        return values

    # ---- tables --------------------------------------------------------
    def rate_tables(self):
        """``{dataset name: float64 array}`` in the reference's dataset naming:
        ``<reaction>`` and ``<action>_<table>`` (chemical_network.py:310-318)."""
        out = {}
        for rxn in sorted(self.reactions.values()):
            out[rxn.name] = np.asarray(rxn.coeff_fn(self), dtype=np.float64)
        for action in sorted(self.cooling_actions.values()):
            for tab in action.tables:
                out["%s_%s" % (action.name, tab)] = np.asarray(
                    action.tables[tab](self), dtype=np.float64)
        return out

    # ---- code generation ----------------------------------------------
    def write_solver(self, solver_name, solver_template="rates_and_rate_tables",
                     ode_solver_source="BE_chem_solve.C", output_dir=".",
                     init_values=None, main_name="main", input_is_number=False):
        """Render the GB300 solver for this network into ``output_dir``.

        Writes ``<name>_solver.cu`` (device functions + kernels + the C
        entry points), ``<name>_solver.h`` (drop-in C header),
        ``<name>_solver_main.cu`` (stand-alone driver), ``<name>_solver_run.py``
        (``run_<name>`` / ``main_run_<name>`` of the reference's Cython module,
        over ctypes), ``<name>_solver_main.py``, ``<name>_tables.dgt``
        (rate/cooling tables) and, when ``init_values`` is given,
        ``<name>_initial_conditions.dgt`` -- the reference's file set with the
        Cython and HDF5 pieces replaced.
        ``solver_template`` selects a template family by name, as in the
        reference (chemical_network.py:285-293); the reference's name maps
        to this package's CUDA family.  ``ode_solver_source`` is accepted for
        signature compatibility: the Newton engine ships with the package.
        """
        from .codegen import render_solver
        from .tablefile import write_table_file
        self.input_is_number = input_is_number
        os.makedirs(output_dir, exist_ok=True)
        paths = render_solver(self, solver_name, output_dir,
                              family=solver_template)
        tpath = os.path.join(output_dir, "%s_tables.dgt" % solver_name)
        write_table_file(tpath, self.rate_tables())
        paths.append(tpath)
        if init_values is not None:
            ipath = os.path.join(output_dir, "%s_initial_conditions.dgt" % solver_name)
            write_table_file(ipath, {k: np.asarray(v, dtype=np.float64)
                                     for k, v in init_values.items()})
            paths.append(ipath)
        return paths
