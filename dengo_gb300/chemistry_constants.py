"""Physical constants used by the rate fits and the generated solvers.

The values are the ones the reference network code uses
(dengo/chemistry_constants.py:26-29); they enter table values and the
mass/number-density conversions, so they are kept identical.
"""

#: Kelvin per electron-volt used to form T_eV = T / tevk.
tevk = 1.1605e4
#: Floor value assigned to rates outside their fitted range.
tiny = 1e-30
#: Hydrogen mass [g] used in every density conversion.
mh = 1.67e-24
#: Boltzmann constant [erg/K] used by initial-condition helpers.
kboltz = 1.380e-16
