"""sympy -> C / CUDA printers for the generated solvers.

``ccode_ref`` is sympy's C99 printer exactly as the reference calls it
(``sympy.printing.ccode``, dengo/chemical_network.py:33,145,151,168): its text
is the host C the reference emits.

``DeviceCodePrinter`` prints the *same* expression tree with the same
operand order, so a CUDA build with ``--fmad=false`` performs the same IEEE
operations in the same order as the host build with ``-ffp-contract=off``.
It differs in three ways only:

* symbols lose their ``[i]`` strip index (the device code holds one cell's
  rates in scalars);
* ``pow(x, n)`` for an integer ``n >= 2`` becomes ``dg_ipow<n>(x)``, this
  package's integer power (exact square; compensated products for higher
  powers).  glibc's ``pow(x, 2)`` equals ``x*x`` for every finite ``x``, so the
  square matches the reference bit for bit; cubes agree except when the exact
  value lies within about 2e-3 ulp of a rounding midpoint;
* other powers call the device ``pow``.
"""

import sympy
from sympy.printing.c import C99CodePrinter


def ccode_ref(expr, assign_to=None):
    """The reference's printer: ``sympy.ccode`` with its defaults."""
    return sympy.ccode(expr, assign_to=assign_to)


class DeviceCodePrinter(C99CodePrinter):
    """C99 printer for ``__device__`` code of one cell."""

    def _print_Symbol(self, expr):
        return super()._print_Symbol(expr).replace("[i]", "")

    def _print_Pow(self, expr):
        e = expr.exp
        if e.is_Integer and int(e) >= 2:
            return "dg_ipow<%d>(%s)" % (int(e), self._print(expr.base))
        return super()._print_Pow(expr)


class FloatDeviceCodePrinter(DeviceCodePrinter):
    """The same expression in FP32: every floating literal is a float
    literal (``1.0f``), rational coefficients are float quotients, and
    other powers call ``powf``; integer coefficients stay integers (they
    convert exactly)."""

    def _print_Float(self, expr):
        return super()._print_Float(expr) + "f"

    def _print_Rational(self, expr):
        return "%d.0f/%d.0f" % (expr.p, expr.q)

    def _print_Pow(self, expr):
        e = expr.exp
        if e.is_Integer and int(e) >= 2:
            return "dg_ipow<%d>(%s)" % (int(e), self._print(expr.base))
        if e == -1:
            return "1.0f/%s" % self.parenthesize(expr.base, sympy.printing.precedence.PRECEDENCE["Pow"])
        return "powf(%s, %s)" % (self._print(expr.base), self._print(e))


def ccode_device32(expr, assign_to=None):
    """``expr`` for the FP32 Jacobian of the mixed-precision solve."""
    printer = FloatDeviceCodePrinter()
    if assign_to is not None and isinstance(assign_to, str):
        assign_to = sympy.Symbol(assign_to)
    return printer.doprint(expr, assign_to=assign_to)


def ccode_device(expr, assign_to=None):
    """Print ``expr`` for the device: same operation order as ``ccode_ref``."""
    printer = DeviceCodePrinter()
    if assign_to is not None and isinstance(assign_to, str):
        assign_to = sympy.Symbol(assign_to)
    return printer.doprint(expr, assign_to=assign_to)


def strip_index(name):
    """Table/rate symbol name without the ``[i]`` suffix."""
    return name.replace("[i]", "")
