"""Atomic numbers and standard atomic weights for the light elements.

The generator reads each element's weight when an ``AtomicSpecies`` is
created (reference: dengo/periodic_table.py:24-40 loads the same three
fields from a CSV).  Weights enter the generated code as literal constants
(mass <-> number density conversion, the mass density in the temperature
formula), so the values below equal the reference's for every element listed.
"""

# (atomic number, standard atomic weight, element name) keyed by symbol.
_ELEMENTS = (
    ("H", 1, 1.00794, "Hydrogen"),
    ("He", 2, 4.002602, "Helium"),
    ("Li", 3, 6.941, "Lithium"),
    ("Be", 4, 9.012182, "Beryllium"),
    ("B", 5, 10.811, "Boron"),
    ("C", 6, 12.0107, "Carbon"),
    ("N", 7, 14.0067, "Nitrogen"),
    ("O", 8, 15.9994, "Oxygen"),
    ("F", 9, 18.9994, "Fluorine"),
    ("Ne", 10, 20.1797, "Neon"),
    ("Na", 11, 22.98976928, "Sodium"),
    ("Mg", 12, 24.305, "Magnesium"),
    ("Al", 13, 26.9815386, "Aluminium"),
    ("Si", 14, 28.0855, "Silicon"),
    ("P", 15, 30.973762, "Phosphorus"),
    ("S", 16, 32.065, "Sulphur"),
    ("Cl", 17, 35.453, "Chlorine"),
    ("Ar", 18, 39.948, "Argon"),
    ("K", 19, 39.0983, "Potassium"),
    ("Ca", 20, 40.078, "Calcium"),
    ("Sc", 21, 44.955912, "Scandium"),
    ("Ti", 22, 47.867, "Titanium"),
    ("V", 23, 50.9415, "Vanadium"),
    ("Cr", 24, 51.9961, "Chromium"),
    ("Mn", 25, 54.938045, "Manganese"),
    ("Fe", 26, 55.845, "Iron"),
    ("Co", 27, 58.933195, "Cobalt"),
    ("Ni", 28, 58.6934, "Nickel"),
    ("Cu", 29, 63.546, "Copper"),
    ("Zn", 30, 65.38, "Zinc"),
)

periodic_table_by_name = {sym: (num, w, name) for sym, num, w, name in _ELEMENTS}
periodic_table_by_number = {num: (w, sym, name) for sym, num, w, name in _ELEMENTS}
