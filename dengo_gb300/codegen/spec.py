"""Flatten a ``ChemicalNetwork`` into what the code templates need.

Orders follow the reference's generated code exactly:

* species: ``sorted(required_species)`` (rates_and_rate_tables.C.template:323);
* tables: reactions by name, then each cooling action by name with its
  tables by name (rates_and_rate_tables.h.template:57-80,
  rates_and_rate_tables.C.template:402-453).  Reactions whose name contains
  ``pi`` and actions whose name contains ``ph`` are tabulated in redshift,
  all others in log T;
* Jacobian: column (variable) major, ``J[var*N + eq]``
  (rates_and_rate_tables.C.template:578-594).
"""

import re
from dataclasses import dataclass, field

import sympy

from .printers import ccode_device, ccode_device32, ccode_ref


@dataclass
class SpeciesSpec:
    index: int
    name: str
    weight: str          # literal as the reference's template prints it
    free_electrons: str  # literal; "0.0" for ge/de
    is_ge: bool
    is_de: bool

    @property
    def counts_in_mdensity(self):
        # rates_and_rate_tables.C.template:496-499
        return self.name not in ("ge", "de", "us_e_0")


@dataclass
class TableSpec:
    index: int
    name: str            # C identifier used by the expressions, e.g. k01, ceHI_ceHI
    kind: str            # "rate" or "cool"
    zdep: bool           # tabulated in redshift instead of log T


@dataclass
class NetworkSpec:
    name: str
    species: list
    tables: list
    T_bounds: tuple      # literals
    nT: int              # table length in T (nbins + 1)
    z_bounds: tuple
    nz: int
    input_is_number: bool
    mass_density_ref: str
    mass_density_dev: str
    T_ref: str
    T_dev: str
    Tge_ref: str
    Tge_dev: str
    T_dev_div: str       # T_dev with x/(gamma - 1.0) as dg_div(x, gm1, rgm1)
    Tge_dev_div: str
    rhs_ref: list        # per species, "rhs[j] = ...;"
    rhs_dev: list        # per species, "f[k] = ...;"
    jac_ref: list        # [var][eq] "Joutput[j] = ...;"
    jac_dev: list        # [var][eq] device statement or None for a structural zero
    jac_dev32: list = field(default_factory=list)     # the same in FP32
    jac_nonzero: list = field(default_factory=list)   # [var][eq] bool
    # Work split of one Newton sweep over NP cooperating warps: part index of
    # every RHS row and every Jacobian entry, {NP: ...}, balanced by sympy
    # operation count (longest-first greedy).
    rhs_part: dict = field(default_factory=dict)      # {NP: [part per row]}
    jac_part: dict = field(default_factory=dict)      # {NP: [var][eq] part}
    stop_time: str = "3.1557e13"   # literal: the network's stop_time (the main driver's dtf)
    write_intermediate: bool = False  # the network's write_intermediate_solutions
    # integer basis of the linear combinations of species the reactions
    # conserve (left null space of the stoichiometry), one list of N
    # coefficients per invariant (0 for ge)
    conservation: list = field(default_factory=list)
    # T(ge) in lane-parallel parts (temperature_lanes), or None when the
    # printed expressions are not of that form
    t_lanes: object = None
    # the RHS rows and Jacobian entries that are flat sums of signed
    # products, as term tables for lane-parallel evaluation (sop_tables)
    sop: object = None

    @property
    def N(self):
        return len(self.species)

    @property
    def NT(self):
        return len(self.tables)

    @property
    def ige(self):
        return [s.index for s in self.species if s.is_ge][0]

    @property
    def ide(self):
        d = [s.index for s in self.species if s.is_de]
        return d[0] if d else -1

    @property
    def has_z_tables(self):
        return any(t.zdep for t in self.tables)

    def nnz(self):
        return sum(sum(1 for v in col if v) for col in self.jac_nonzero)

    def jac_col_mask(self, var):
        """Bit q set when d rhs_q / d y_var is structurally nonzero."""
        return sum(1 << q for q, v in enumerate(self.jac_nonzero[var]) if v)


_GAMMA_DIV = re.compile(r"\b([A-Za-z_][A-Za-z0-9_]*)/\(gamma - 1\.0\)")


def gamma_div(text):
    """Rewrite ``x/(gamma - 1.0)`` as ``dg_div(x, gm1, rgm1)`` (same value)."""
    return _GAMMA_DIV.sub(r"dg_div(\1, gm1, rgm1)", text)


_DTERM = re.compile(r"^(?:(\d+\.\d*(?:e[+-]?\d+)?)\*)?([A-Za-z_][A-Za-z0-9_]*)$")


def temperature_lanes(species, mass_density, T_div, Tge_div):
    """The temperature as lane-parallel parts: ``{"density": [(species
    index, weight literal), ...], "quot": [species index, ...]}`` when the
    printed expressions are ``density = w_0*y_a + w_1*y_b + ...`` and
    ``T = density*ge*mh/(kb*(dg_div(y_c, gm1, rgm1) + ...))`` (``Tge`` the
    same without ``*ge``), each sum in the order listed; else None.  Every
    term is one product or one quotient and the sums run left to right, so
    terms formed on separate lanes and summed in that order give the
    printed expressions' values bit for bit."""
    index = {sp.name: sp.index for sp in species}
    dens = []
    for term in mass_density.split(" + "):
        m = _DTERM.match(term.strip())
        if not m or m.group(2) not in index:
            return None
        dens.append((index[m.group(2)], m.group(1) or "1.0"))
    quot = []
    inner = None
    for pre in ("density*ge*mh/(kb*(", "density*mh/(kb*("):
        text = T_div if "ge*" in pre else Tge_div
        if not (text.startswith(pre) and text.endswith("))")):
            return None
        body = text[len(pre):-2]
        if inner is None:
            inner = body
        elif body != inner:
            return None
    for term in inner.split(" + "):
        m = re.match(r"^dg_div\(([A-Za-z_][A-Za-z0-9_]*), gm1, rgm1\)$", term.strip())
        if not m or m.group(1) not in index:
            return None
        quot.append(index[m.group(1)])
    if not dens or not quot or len(dens) > 32 or len(quot) > 32:
        return None
    return {"density": dens, "quot": quot}


_SOP_TOK = re.compile(r"\s*(?:(dg_ipow<(\d+)>\(([A-Za-z_][A-Za-z0-9_]*)\))|"
                      r"(\d+\.\d*(?:e[+-]?\d+)?|\d+(?:e[+-]?\d+)?)|([A-Za-z_][A-Za-z0-9_]*)|([-+*]))")


def sop_parse(expr, names):
    """``[(sign, [factor, ...]), ...]`` when the C expression ``expr`` is a
    flat sum of signed products of atoms -- ``[-]a*b*c +|- d*e ...`` with
    atoms numeric literals, names in ``names`` (rates, species) and
    ``dg_ipow<n>(species)`` -- else None.  C evaluates such an expression as
    ((t0 + t1) - t2) ..., each term as ((a*b)*c)...; a leading unary minus
    binds to the first factor, which negates the term exactly.  Factors:
    ``("lit", text)``, ``("name", name)``, ``("pow", n, name)``."""
    toks, pos, e = [], 0, expr.strip()
    while pos < len(e):
        m = _SOP_TOK.match(e, pos)
        if not m or m.end() == pos:
            return None
        pos = m.end()
        if m.group(1):
            if m.group(3) not in names or not 2 <= int(m.group(2)) <= 6:
                return None
            toks.append(("pow", int(m.group(2)), m.group(3)))
        elif m.group(4):
            toks.append(("lit", m.group(4)))
        elif m.group(5):
            if m.group(5) not in names:
                return None
            toks.append(("name", m.group(5)))
        else:
            toks.append(m.group(6))
    terms, i, sign = [], 0, 1
    if toks and toks[0] == "-":
        sign, i = -1, 1
    while True:
        facs = []
        while True:
            if i >= len(toks) or isinstance(toks[i], str):
                return None
            facs.append(toks[i])
            i += 1
            if i < len(toks) and toks[i] == "*":
                i += 1
                continue
            break
        terms.append((sign, facs))
        if i == len(toks):
            return terms
        if toks[i] not in ("+", "-"):
            return None
        sign = 1 if toks[i] == "+" else -1
        i += 1


def sop_tables(species, tables, rhs_dev, jac_dev, jac_nz):
    """Operand and term tables of the RHS rows and Jacobian entries that
    sop_parse accepts, for lane-parallel evaluation (the wide engine), and
    the lists of the others.  Operands: the rates, the species, the powers
    dg_ipow<n>(species) that occur, the literals, and 1.0 (which pads a
    term's factors: x * 1.0 is x).  A term is a sign and FMAX operand
    indices; an entry is a term range and a final operation (RHS ge row:
    / mdensity; Jacobian: dg_div by mdensity for the ge row, * Tge for the ge
    column).  None when nothing parses."""
    sp_index = {sp.name: sp.index for sp in species}
    ge = [sp.index for sp in species if sp.is_ge][0]
    names = set(sp_index) | {t.name for t in tables}
    t_index = {t.name: t.index for t in tables}
    NT, N = len(tables), len(species)

    def body(stmt, lhs):
        m = re.match(r"^\s*%s = (.*);\s*$" % re.escape(lhs), stmt, re.S)
        return m.group(1) if m else None

    rhs, jac = {}, {}
    for i in range(N):
        b = body(rhs_dev[i], "f[%d]" % i)
        t = sop_parse(b, names) if b is not None else None
        if t is not None:
            rhs[i] = t
    for v in range(N):
        for q in range(N):
            if not jac_nz[v][q]:
                continue
            b = body(jac_dev[v][q], "jv")
            t = sop_parse(b, names) if b is not None else None
            if t is not None:
                jac[(q, v)] = t
    if not rhs and not jac:
        return None
    pows = sorted({(f[1], sp_index[f[2]]) for ts in list(rhs.values()) + list(jac.values())
                   for _, fs in ts for f in fs if f[0] == "pow"})
    lits = []
    for ts in list(rhs.values()) + list(jac.values()):
        for _, fs in ts:
            for f in fs:
                if f[0] == "lit" and f[1] not in lits:
                    lits.append(f[1])
    op_pow = {p: NT + N + k for k, p in enumerate(pows)}
    op_lit = {l: NT + N + len(pows) + k for k, l in enumerate(lits)}
    one = NT + N + len(pows) + len(lits)
    fmax = max(len(fs) for ts in list(rhs.values()) + list(jac.values()) for _, fs in ts)

    def operand(f):
        if f[0] == "lit":
            return op_lit[f[1]]
        if f[0] == "pow":
            return op_pow[(f[1], sp_index[f[2]])]
        return t_index[f[1]] if f[1] in t_index else NT + sp_index[f[1]]

    def flatten(entries):
        terms, ranges = [], []
        for key, ts in entries:
            t0 = len(terms)
            for sign, fs in ts:
                ops = [operand(f) for f in fs]
                terms.append((sign, ops + [one] * (fmax - len(ops))))
            ranges.append((key, t0, len(terms)))
        return terms, ranges

    rhs_terms, rhs_ranges = flatten(sorted(rhs.items()))
    jac_terms, jac_ranges = flatten(sorted(jac.items(), key=lambda kv: (kv[0][1], kv[0][0])))

    def lit_value(text):
        return text if ("." in text or "e" in text) else text + ".0"

    rhs_rest = [i for i in range(N) if i not in rhs]
    jac_rest = [(q, v) for v in range(N) for q in range(N) if jac_nz[v][q] and (q, v) not in jac]
    # the other rows / entries as scalar code on up to three warps, balanced
    # by the length of their printed expressions
    rk, jk = min(3, len(rhs_rest)), min(3, len(jac_rest))
    rpart = dict(zip(rhs_rest, balance([float(len(rhs_dev[i])) for i in rhs_rest], rk))) \
        if rk else {}
    jpart = dict(zip(jac_rest, balance([float(len(jac_dev[v][q])) for q, v in jac_rest], jk))) \
        if jk else {}
    enc = lambda terms: [(ops[0] | (0x8000 if sign < 0 else 0), *ops[1:]) for sign, ops in terms]
    return {"nops": one + 1, "one": one, "fmax": fmax, "pows": pows,
            "rk": rk, "jk": jk, "rhs_rest_part": rpart, "jac_rest_part": jpart,
            "rhs_enc": enc(rhs_terms), "jac_enc": enc(jac_terms),
            "lits": [lit_value(l) for l in lits], "lit0": NT + N + len(pows),
            "rhs_terms": rhs_terms,
            "rhs_entries": [(i, t0, t1, 1 if i == ge else 0) for i, t0, t1 in rhs_ranges],
            "rhs_rest": rhs_rest,
            "jac_terms": jac_terms,
            "jac_entries": [(q, v, t0, t1, (1 if q == ge else 0) | (2 if v == ge else 0))
                            for (q, v), t0, t1 in jac_ranges],
            "jac_rest": jac_rest}


_CX_TOK = re.compile(r"\s*(dg_ipow<\d+>|dg_div|[A-Za-z_][A-Za-z0-9_]*|"
                     r"\d+\.\d*(?:e[+-]?\d+)?|\d+(?:e[+-]?\d+)?|[-+*/(),])")


def _cx_parse(text):
    """Expression tree of a printed C expression (nested tuples), or None."""
    toks, pos = [], 0
    text = text.strip()
    while pos < len(text):
        m = _CX_TOK.match(text, pos)
        if not m or m.end() == pos:
            return None
        toks.append(m.group(1))
        pos = m.end()
    i = [0]

    def peek():
        return toks[i[0]] if i[0] < len(toks) else None

    def take():
        i[0] += 1
        return toks[i[0] - 1]

    def expr():
        n = term()
        while peek() in ("+", "-"):
            op = take()
            n = (op, n, term())
        return n

    def term():
        n = unary()
        while peek() in ("*", "/"):
            op = take()
            n = (op, n, unary())
        return n

    def unary():
        if peek() == "-":
            take()
            return ("neg", unary())
        return atom()

    def atom():
        x = take()
        if x == "(":
            n = expr()
            take()
            return n
        if peek() == "(":
            take()
            args = [expr()]
            while peek() == ",":
                take()
                args.append(expr())
            take()
            return ("call", x, tuple(args))
        return ("leaf", x)

    try:
        n = expr()
    except IndexError:
        return None
    return n if i[0] == len(toks) else None


def _cx_nodes(n, acc):
    """The operation nodes of tree n with their FP64 cost (a division 9, a
    dg_div 3, a cube or other power 6, other calls 20)."""
    if n[0] == "leaf" or n in acc:
        return
    if n[0] == "neg":
        _cx_nodes(n[1], acc)
        return
    if n[0] == "call":
        name = n[1]
        acc[n] = 3 if name == "dg_div" else (1 if name == "dg_ipow<2>" else
                                             (6 if name.startswith("dg_ipow") else 20))
        for a in n[2]:
            _cx_nodes(a, acc)
        return
    acc[n] = 9 if n[0] == "/" else 1
    _cx_nodes(n[1], acc)
    _cx_nodes(n[2], acc)


def balance_shared(texts, nparts):
    """Part index for each statement: longest-first greedy onto the part
    whose resulting cost is lowest, where a part's cost counts each
    operation of its statements' expressions once -- the compiler computes
    a subexpression several statements of one part share only once -- so
    statements that share large subexpressions (the ge row's cooling terms)
    end up together.  None texts (structural zeros) cost 0.5."""
    nodes = []
    for t in texts:
        if t is None:
            nodes.append(None)
            continue
        m = re.match(r"^\s*[A-Za-z_][A-Za-z0-9_\[\]]* = (.*?);", t, re.S)
        tree = _cx_parse(m.group(1)) if m else None
        acc = {}
        if tree is not None:
            _cx_nodes(tree, acc)
        else:
            acc[("text", t)] = float(len(t)) / 8.0
        nodes.append(acc)
    own = [0.5 if a is None else sum(a.values()) + 4.0 for a in nodes]
    sets = [dict() for _ in range(nparts)]
    loads = [0.0] * nparts
    part = [0] * len(texts)
    for k in sorted(range(len(texts)), key=lambda k: (-own[k], k)):
        best = None
        for p in range(nparts):
            if nodes[k] is None:
                new = loads[p] + 0.5
            else:
                extra = sum(c for n, c in nodes[k].items() if n not in sets[p])
                new = loads[p] + extra + 4.0
            key = (max([new] + [loads[q] for q in range(nparts) if q != p]), new, p)
            if best is None or key < best[0]:
                best = (key, p, new)
        _, p, new = best
        part[k] = p
        loads[p] = new
        if nodes[k] is not None:
            sets[p].update(nodes[k])
    return part


def balance(costs, nparts):
    """Part index for each item: longest-first greedy onto the least-loaded
    part (ties to the lowest part), so parts carry similar operation counts."""
    load = [0.0] * nparts
    part = [0] * len(costs)
    for i in sorted(range(len(costs)), key=lambda i: (-costs[i], i)):
        p = min(range(nparts), key=lambda k: (load[k], k))
        part[i] = p
        load[p] += costs[i]
    return part


def _lit(v):
    """The text Jinja prints for a Python number (``str``), as the reference's
    templates do for weights, charges and bounds."""
    return str(v)


def conservation_basis(net, ordered):
    """Integer basis of the species combinations every reaction conserves:
    the null space of the stoichiometry matrix (reactions x species, ge
    excluded), each vector scaled to coprime integers.  For the primordial
    network these are the H and He nuclei; the reference's k12
    (H2 + e -> 2 H+ + e, dengo/primordial_rates.py:191) does not conserve
    charge, so charge is not among them, while the ion-by-ion networks also
    conserve a charge combination."""
    chem = [s.name for s in ordered if s.name != "ge"]
    rows = []
    for rn in sorted(net.reactions):
        r = net.reactions[rn]
        rows.append([sympy.nsimplify(sum(n for n, x in r.right_side if x.name == c) -
                                     sum(n for n, x in r.left_side if x.name == c))
                     for c in chem])
    if not rows:
        return []
    out = []
    for v in sympy.Matrix(rows).nullspace():
        den = sympy.ilcm(*[sympy.fraction(x)[1] for x in v])
        ints = [int(x * den) for x in v]
        g = 0
        for x in ints:
            g = sympy.igcd(g, x)
        ints = [x // g for x in ints]
        if sum(ints) < 0:
            ints = [-x for x in ints]
        full = iter(ints)
        out.append([0 if s.name == "ge" else next(full) for s in ordered])
    return out


def network_spec(net, name):
    species = []
    for i, s in enumerate(sorted(net.required_species)):
        species.append(SpeciesSpec(
            index=i, name=s.name, weight=_lit(s.weight),
            free_electrons=_lit(getattr(s, "free_electrons", 0.0)),
            is_ge=(s.name == "ge"), is_de=(s.name in ("de", "us_e_0"))))
    tables = []
    for rname in sorted(net.reactions):
        tables.append(TableSpec(len(tables), rname, "rate", "pi" in rname))
    for cname in sorted(net.cooling_actions):
        for tname in sorted(net.cooling_actions[cname].tables):
            tables.append(TableSpec(len(tables), "%s_%s" % (cname, tname), "cool",
                                    "ph" in cname))
    ordered = sorted(net.required_species)
    rhs_ref, rhs_dev = [], []
    for i, s in enumerate(ordered):
        e = net.rhs_expression(s)
        rhs_ref.append(ccode_ref(e, assign_to=sympy.Symbol("rhs[j]")))
        rhs_dev.append(ccode_device(e, assign_to=sympy.Symbol("f[%d]" % i)))
    rhs_cost = [float(sympy.count_ops(net.rhs_expression(s))) + 1.0 for s in ordered]
    jac_ref, jac_dev, jac_dev32, jac_nz, jac_cost = [], [], [], [], []
    for v, s1 in enumerate(ordered):
        cr, cd, cd32, cn = [], [], [], []
        for q, s2 in enumerate(ordered):
            e = net.jacobian_expression(s2, s1)
            cr.append(ccode_ref(e, assign_to=sympy.Symbol("Joutput[j]")))
            nz = not (e == 0)
            cn.append(nz)
            cd.append(ccode_device(e, assign_to=sympy.Symbol("jv")) if nz else None)
            cd32.append(ccode_device32(e, assign_to=sympy.Symbol("jv")) if nz else None)
            jac_cost.append(float(sympy.count_ops(e)) + 4.0 if nz else 0.5)
        jac_ref.append(cr)
        jac_dev.append(cd)
        jac_dev32.append(cd32)
        jac_nz.append(cn)
    N = len(ordered)
    rhs_part, jac_part = {}, {}
    for npart in (1, 2, 4):
        rhs_part[npart] = balance(rhs_cost, npart)
        flat = balance_shared([jac_dev[v][q] for v in range(N) for q in range(N)], npart) \
            if npart > 1 else balance(jac_cost, npart)
        jac_part[npart] = [flat[v * N:(v + 1) * N] for v in range(N)]
    md = net.mass_density_expression()
    T = net.temperature_expression(False)
    Tg = net.temperature_expression(True)
    z = getattr(net, "z", None)
    return NetworkSpec(
        name=name, species=species, tables=tables,
        T_bounds=(_lit(net.T_bounds[0]), _lit(net.T_bounds[1])),
        nT=len(net.T),
        z_bounds=(_lit(net.z_bounds[0]), _lit(net.z_bounds[1])),
        nz=(len(z) if z is not None else 0),
        input_is_number=bool(getattr(net, "input_is_number", False)),
        stop_time=repr(float(net.stop_time)),
        write_intermediate=bool(getattr(net, "write_intermediate_solutions", False)),
        conservation=conservation_basis(net, ordered),
        mass_density_ref=ccode_ref(md), mass_density_dev=ccode_device(md),
        T_ref=ccode_ref(T), T_dev=ccode_device(T),
        Tge_ref=ccode_ref(Tg), Tge_dev=ccode_device(Tg),
        T_dev_div=gamma_div(ccode_device(T)), Tge_dev_div=gamma_div(ccode_device(Tg)),
        t_lanes=temperature_lanes(species, ccode_device(md), gamma_div(ccode_device(T)),
                                  gamma_div(ccode_device(Tg))),
        sop=sop_tables(species, tables, rhs_dev, jac_dev, jac_nz),
        rhs_ref=rhs_ref, rhs_dev=rhs_dev,
        jac_ref=jac_ref, jac_dev=jac_dev, jac_dev32=jac_dev32, jac_nonzero=jac_nz,
        rhs_part=rhs_part, jac_part=jac_part)
