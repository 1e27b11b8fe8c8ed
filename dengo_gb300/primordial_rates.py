"""Primordial H/He/H2 chemistry: 8 species and 22 reactions (k01-k19, k21-k23).

The rate fits are the published ones the reference tabulates
(dengo/primordial_rates.py:35-294; Abel et al. 1997, Glover & Abel 2008).
Each table is evaluated with the same numpy operations in the same order
(``c0 + c1*x + c2*x**2 + ...`` term by term, piecewise branches applied by
boolean masks in the same sequence), so the tables are bit-identical to the
reference's on the same machine.
"""

import numpy as np

from .chemistry_constants import tiny
from .reaction_classes import (AtomicSpecies, MolecularSpecies, reaction,
                               registry_setup, species_registry)


def _series(x, coeffs):
    """``coeffs[0] + coeffs[1]*x + coeffs[2]*x**2 + ...``, left to right."""
    acc = coeffs[0] + coeffs[1] * x
    for k in range(2, len(coeffs)):
        acc = acc + coeffs[k] * x**k
    return acc


# ln(rate) polynomial fits in ln(T_eV).
_K01 = (-32.71396786375, 13.53655609057, -5.739328757388, 1.563154982022,
        -0.2877056004391, 0.03482559773736999, -0.00263197617559,
        0.0001119543953861, -2.039149852002e-6)
_K02 = (-28.61303380689232, -0.7241125657826851, -0.02026044731984691,
        -0.002380861877349834, -0.0003212605213188796, -0.00001421502914054107,
        4.989108920299513e-6, 5.755614137575758e-7, -1.856767039775261e-8,
        -3.071135243196595e-9)
_K03 = (-44.09864886561001, 23.91596563469, -10.75323019821, 3.058038757198,
        -0.5685118909884001, 0.06795391233790001, -0.005009056101857001,
        0.0002067236157507, -3.649161410833e-6)
_K05 = (-68.71040990212001, 43.93347632635, -18.48066993568, 4.701626486759002,
        -0.7692466334492, 0.08113042097303, -0.005324020628287001,
        0.0001975705312221, -3.165581065665e-6)
_K08 = (-20.06913897587003, 0.2289800603272916, 0.03599837721023835,
        -0.004555120027032095, -0.0003105115447124016, 0.0001073294010367247,
        -8.36671960467864e-6, 2.238306228891639e-7)
_K11 = (-24.24914687731536, 3.400824447095291, -3.898003964650152,
        2.045587822403071, -0.5416182856220388, 0.0841077503763412,
        -0.007879026154483455, 0.0004138398421504563, -9.36345888928611e-6)
_K14 = (-18.01849334273, 2.360852208681, -0.2827443061704, 0.01623316639567,
        -0.03365012031362999, 0.01178329782711, -0.001656194699504,
        0.0001068275202678, -2.631285809207e-6)
_K15 = (-20.37260896533324, 1.139449335841631, -0.1421013521554148,
        0.00846445538663, -0.0014327641212992, 0.0002012250284791,
        0.0000866396324309, -0.00002585009680264, 2.4555011970392e-6,
        -8.06838246118e-8)


def _he_recombination(tev):
    """Radiative + dielectronic recombination fit shared by k02 (T <= 5500 K)
    and k04."""
    return (1.54e-9 * (1. + 0.3 / np.exp(8.099328789667 / tev))
            / (np.exp(40.49664394833662 / tev) * tev**1.5)
            + 3.92e-13 / tev**0.6353)


@registry_setup
def setup_primordial():
    """Register the primordial species and reactions; returns the new names."""
    HI = AtomicSpecies("H", 0.0)
    HII = AtomicSpecies("H", 1.0)
    HeI = AtomicSpecies("He", 0.0)
    HeII = AtomicSpecies("He", 1.0)
    HeIII = AtomicSpecies("He", 2.0)
    HM = AtomicSpecies("H", -1.0)
    H2I = MolecularSpecies("H2", 2.0, 0.0)
    H2II = MolecularSpecies("H2", 2.0, 1.0)
    de = species_registry["de"]

    @reaction("k01", [(1, HI), (1, de)], [(1, HII), (2, de)])
    def k01(state):
        return np.exp(_series(state.logtev, _K01))

    @reaction("k02", [(1, HII), (1, de)], [(1, HI)])
    def k02(state):
        cold = ~(state.T > 5500)
        vals = np.exp(_series(state.logtev, _K02))
        vals[cold] = _he_recombination(state.tev[cold])
        low = state.tev < 0.8
        vals[low] = 3.92e-13 / state.tev[low]**0.6353
        return vals

    @reaction("k03", [(1, HeI), (1, de)], [(1, HeII), (2, de)])
    def k03(state):
        cold = ~(state.tev > 0.8)
        vals = np.exp(_series(state.logtev, _K03))
        vals[cold] = tiny
        return vals

    @reaction("k04", [(1, HeII), (1, de)], [(1, HeI)])
    def k04(state):
        cold = ~(state.tev > 0.8)
        vals = _he_recombination(state.tev)
        vals[cold] = tiny
        return vals

    @reaction("k05", [(1, HeII), (1, de)], [(1, HeIII), (2, de)])
    def k05(state):
        cold = ~(state.tev > 0.8)
        vals = np.exp(_series(state.logtev, _K05))
        vals[cold] = tiny
        return vals

    @reaction("k06", [(1, HeIII), (1, de)], [(1, HeII)])
    def k06(state):
        return (3.36e-10 / np.sqrt(state.T) / (state.T / 1.e3)**0.2
                / (1 + (state.T / 1.e6)**0.7))

    @reaction("k07", [(1, HI), (1, de)], [(1, HM)])
    def k07(state):
        return 6.77e-15 * state.tev**0.8779

    @reaction("k08", [(1, HM), (1, HI)], [(1, H2I), (1, de)])
    def k08(state):
        cold = ~(state.tev > 0.1)
        vals = np.exp(_series(state.logtev, _K08))
        vals[cold] = 1.43e-9
        return vals

    @reaction("k09", [(1, HI), (1, HII)], [(1, H2II)])
    def k09(state):
        hot = state.T > 6.7e3
        vals = 1.85e-23 * state.T**1.8
        vals[hot] = 5.81e-16 * (state.T[hot] / 56200)**(
            -0.6657 * np.log10(state.T[hot] / 56200))
        return vals

    @reaction("k10", [(1, H2II), (1, HI)], [(1, H2I), (1, HII)])
    def k10(state):
        return state.T * 0.0 + 6.0e-10

    @reaction("k11", [(1, H2I), (1, HII)], [(1, H2II), (1, HI)])
    def k11(state):
        cold = ~(state.tev > 0.3)
        vals = np.exp(_series(state.logtev, _K11))
        vals[cold] = tiny
        return vals

    @reaction("k12", [(1, H2I), (1, de)], [(2, HII), (1, de)])
    def k12(state):
        return 5.6e-11 * np.exp(-102124 / state.T) * state.T**0.5

    @reaction("k13", [(1, H2I), (1, HI)], [(3, HI)])
    def k13(state):
        # Glover (2008) collisional dissociation by H.
        lt = np.log10(state.T)
        return 10.0**(-178.4239 - 68.42243 * np.log10(state.T)
                      + 43.20243 * lt**2
                      - 4.633167 * lt**3
                      + 69.70086 * np.log10(1 + 40870.38 / state.T)
                      - (23705.7 / state.T))

    @reaction("k14", [(1, HM), (1, de)], [(1, HI), (2, de)])
    def k14(state):
        cold = ~(state.tev > 0.04)
        vals = np.exp(_series(state.logtev, _K14))
        vals[cold] = tiny
        return vals

    @reaction("k15", [(1, HM), (1, HI)], [(2, HI), (1, de)])
    def k15(state):
        cold = ~(state.tev > 0.1)
        vals = np.exp(_series(state.logtev, _K15))
        vals[cold] = 2.56e-9 * state.tev[cold]**1.78186
        return vals

    @reaction("k16", [(1, HM), (1, HII)], [(2, HI)])
    def k16(state):
        return 6.5e-9 / np.sqrt(state.tev)

    @reaction("k17", [(1, HM), (1, HII)], [(1, H2II), (1, de)])
    def k17(state):
        hot = ~(state.T < 1e4)
        vals = 1.0e-8 * state.T**(-0.4)
        vals[hot] = 4.0e-4 * state.T[hot]**(-1.4) * np.exp(-15100.0 / state.T[hot])
        return vals

    @reaction("k18", [(1, H2II), (1, de)], [(2, HI)])
    def k18(state):
        cold = ~(state.T > 617)
        vals = 1.32e-6 * state.T**(-0.76)
        vals[cold] = 1.e-8
        return vals

    @reaction("k19", [(1, H2II), (1, HM)], [(1, HI), (1, H2I)])
    def k19(state):
        return 5.e-7 * np.sqrt(100. / state.T)

    @reaction("k21", [(2, HI), (1, H2I)], [(2, H2I)])
    def k21(state):
        return 2.8e-31 * (state.T**(-0.6))

    @reaction("k22", [(2, HI), (1, HI)], [(1, H2I), (1, HI)])
    def k22(state):
        # Glover (2008) three-body H2 formation.
        return 7.7e-31 / state.T**0.464

    @reaction("k23", [(1, H2I), (1, H2I)], [(2, HI), (1, H2I)])
    def k23(state):
        return ((8.125e-8 / np.sqrt(state.T))
                * np.exp(-52000 / state.T)
                * (1.0 - np.exp(-6000 / state.T)))
