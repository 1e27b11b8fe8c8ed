"""Primordial heating/cooling actions (dengo/primordial_cooling.py:34-316).

Each action's equation names the species by their state-vector names
(``H_1`` = H I, ``H_2`` = H II, ``He_2`` = He II, ``H2_1`` = H2, ...).  The
reference's equations use the pre-rename names (``HI``, ``HeII``, ...), which
resolve to the same symbols once aliased; the resulting expressions are
identical.  Tables are evaluated with the reference's numpy operations in
the same order, so they are bit-identical on the same machine.

Importing this module registers the actions, as in the reference.
``compton`` is registered but kept out of the standard primordial network:
its equation depends on the redshift ``z`` and on ``T`` directly.
"""

import numpy as np

from .reaction_classes import cooling_action, reaction_registry

dhuge = 1.0e30


# -- collisional excitation ------------------------------------------------
@cooling_action("ceHI", "-ceHI * H_1 * de")
def _ceHI(eq):
    @eq.table
    def ceHI(state):
        return 7.5e-19 * np.exp(-np.minimum(np.log(dhuge), 118348.0 / state.T)) \
            / (1.0 + np.sqrt(state.T / 1.0e5))


@cooling_action("ceHeI", "-ceHeI * He_2 * de**2")
def _ceHeI(eq):
    @eq.table
    def ceHeI(state):
        return 9.1e-27 * np.exp(-np.minimum(np.log(dhuge), 13179.0 / state.T)) \
            * state.T**(-0.1687) / (1.0 + np.sqrt(state.T / 1.0e5))


@cooling_action("ceHeII", "-ceHeII * He_2 * de")
def _ceHeII(eq):
    @eq.table
    def ceHeII(state):
        return 5.54e-17 * np.exp(-np.minimum(np.log(dhuge), 473638.0 / state.T)) \
            * state.T**(-0.397) / (1. + np.sqrt(state.T / 1.0e5))


# -- collisional ionisation -------------------------------------------------
@cooling_action("ciHeIS", "-ciHeIS*He_2*de**2")
def _ciHeIS(eq):
    @eq.table
    def ciHeIS(state):
        return 5.01e-27 * (state.T)**(-0.1687) / (1. + np.sqrt(state.T / 1.0e5)) \
            * np.exp(-np.minimum(np.log(dhuge), 55338.0 / state.T))


@cooling_action("ciHI", "-ciHI*H_1*de")
def _ciHI(eq):
    @eq.table
    def ciHI(state):
        return 2.18e-11 * reaction_registry["k01"].coeff_fn(state)


@cooling_action("ciHeI", "-ciHeI*He_1*de")
def _ciHeI(eq):
    @eq.table
    def ciHeI(state):
        return 3.94e-11 * reaction_registry["k03"].coeff_fn(state)


@cooling_action("ciHeII", "-ciHeII*He_2*de")
def _ciHeII(eq):
    @eq.table
    def ciHeII(state):
        return 8.72e-11 * reaction_registry["k05"].coeff_fn(state)


# -- recombination ------------------------------------------------------------
def _case_a(T, norm):
    return norm * np.sqrt(T) * (T / 1000.0)**(-0.2) / (1.0 + (T / 1.0e6)**(0.7))


@cooling_action("reHII", "-reHII * H_2 * de")
def _reHII(eq):
    @eq.table
    def reHII(state):
        return _case_a(state.T, 8.70e-27)


@cooling_action("reHeII1", "-reHeII1 * He_2 * de")
def _reHeII1(eq):
    @eq.table
    def reHeII1(state):
        return 1.55e-26 * state.T**0.3647


@cooling_action("reHeII2", "-reHeII2 * He_2 * de")
def _reHeII2(eq):
    @eq.table
    def reHeII2(state):
        return 1.24e-13 * state.T**(-1.5) \
            * np.exp(-np.minimum(np.log(dhuge), 470000.0 / state.T)) \
            * (1. + 0.3 * np.exp(-np.minimum(np.log(dhuge), 94000.0 / state.T)))


@cooling_action("reHeIII", "-reHeIII * He_3 * de")
def _reHeIII(eq):
    @eq.table
    def reHeIII(state):
        return _case_a(state.T, 3.48e-26)


# -- bremsstrahlung -----------------------------------------------------------
@cooling_action("brem", "-brem * (H_2 + He_2 + 4.0*He_3) * de")
def _brem(eq):
    @eq.table
    def brem(state):
        return 1.43e-27 * np.sqrt(state.T) \
            * (1.1 + 0.34 * np.exp(-(5.5 - np.log10(state.T))**2 / 3.0))


# -- H2 rovibrational cooling, Glover & Abel (2008) ---------------------------
def _clip_lt3(T):
    tm = np.maximum(T, 10.0e0)
    tm = np.minimum(tm, 1.e4)
    return np.log10(tm / 1.e3)


def _pow10_series(x, coeffs):
    acc = coeffs[0] + coeffs[1] * x
    for k in range(2, len(coeffs)):
        acc = acc + coeffs[k] * x**k
    return 10**acc


_GA_HI_HOT = (-24.311209e0, 4.6450521e0, -3.7209846e0, 5.9369081e0,
              -5.5108047e0, 1.5538288e0)
_GA_HI_MID = (-24.311209e0, 3.5692468e0, -11.332860e0, -27.850082e0,
              -21.328264e0, -4.2519023e0)
_GA_HI_COLD = (-16.818342e0, 37.383713e0, 58.145166e0, 48.656103e0,
               20.159831e0, 3.8479610e0)
_GA_H2 = (-23.962112e0, 2.09433740e0, -0.77151436e0, 0.43693353e0,
          -0.14913216e0, -0.033638326e0)
_GA_HE = (-23.689237e0, 2.1892372e0, -0.81520438e0, 0.29036281e0,
          -0.16596184e0, 0.19191375e0)
_GA_HP = (-21.716699e0, 1.3865783e0, -0.37915285e0, 0.11453688e0,
          -0.23214154e0, 0.058538864e0)
_GA_EL_HOT = (-22.190316, 1.5728955, -0.21335100, 0.96149759, -0.91023195,
              0.13749749)
_GA_EL_COLD = (-34.286155e0, -48.537163e0, -77.121176e0, -51.352459e0,
               -15.169160e0, -0.98120322e0)


@cooling_action("gloverabel08", "-(H2_1)*gphdl/(1.0+gphdl/galdl)")
def _gloverabel08(eq):
    @eq.table
    def gpldl(state):
        # Galli & Palla (1998) low-density limit (tabulated, unused by the equation).
        tm = np.minimum(np.maximum(state.T, 13.0), 1e5)
        lt = np.log10(tm)
        return 10.**(-103.0 + 97.59 * lt - 48.05 * lt**2 + 10.80 * lt * lt * lt
                     - 0.9032 * lt * lt * lt * lt)

    @eq.table
    def gphdl(state):
        # Hollenbach & McKee (1979) high-density limit.
        tm = np.maximum(state.T, 10.0e0)
        tm = np.minimum(tm, 1.e4)
        t3 = tm / 1000.
        HDLR = ((9.5e-22 * t3**3.76) / (1. + 0.12 * t3**2.1)
                * np.exp(-(0.13 / t3)**3) + 3.e-24 * np.exp(-0.51 / t3))
        HDLV = (6.7e-19 * np.exp(-5.86 / t3) + 1.6e-18 * np.exp(-11.7 / t3))
        return (HDLR + HDLV)

    @eq.table
    def gaHI(state):
        lt3 = _clip_lt3(state.T)
        cold = state.T < 100.0
        mid = state.T < 1000.0
        vals = _pow10_series(lt3, _GA_HI_HOT)
        vals[mid] = _pow10_series(lt3[mid], _GA_HI_MID)
        vals[cold] = _pow10_series(lt3[cold], _GA_HI_COLD)
        return vals

    @eq.table
    def gaH2(state):
        return _pow10_series(_clip_lt3(state.T), _GA_H2)

    @eq.table
    def gaHe(state):
        return _pow10_series(_clip_lt3(state.T), _GA_HE)

    @eq.table
    def gaHp(state):
        return _pow10_series(_clip_lt3(state.T), _GA_HP)

    @eq.table
    def gael(state):
        lt3 = _clip_lt3(state.T)
        cold = state.T < 200
        vals = _pow10_series(lt3, _GA_EL_HOT)
        vals[cold] = _pow10_series(lt3[cold], _GA_EL_COLD)
        return vals

    eq.temporary("galdl", "gaHI*H_1 + gaH2*H2_1 + gaHe*He_1 + gaHp*H_2 + gael*de")


# -- Compton cooling off the CMB (Peebles 1971) -------------------------------
@cooling_action("compton", "-(comp1)*(T - (comp2))*de")
def _compton(eq):
    @eq.table
    def comp(state):
        return 5.65e-36 + state.T * 0.0

    eq.temporary("z", "z")
    eq.temporary("comp1", "comp * (1.0 + z)**4")
    eq.temporary("comp2", "2.73 * (1.0 + z)")
    eq.temporary("T", "T")


# -- dust photoelectric heating (disabled by its 0.0 factor in the reference) -
@cooling_action("gammah", "0.0*gammah * H_1 * H_2")
def _gammah(eq):
    @eq.table
    def gammah(state):
        return 8.5e-26 + state.T


@cooling_action("h2formation", "h2mheat*H_1*H_1*H_1 - h2mcool*H2_1*H_1")
def _h2formation(eq):
    @eq.table
    def h2mheat(state):
        return 7.177e-12 * reaction_registry["k22"].coeff_fn(state)

    @eq.table
    def h2mcool(state):
        return 7.177e-12 * reaction_registry["k13"].coeff_fn(state)
