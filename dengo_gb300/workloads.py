"""Seeded synthetic cell populations for the benchmark configurations.

No public dataset exists for this solver; every workload is drawn here from
``numpy.random.Generator(PCG64(seed))``.

Primordial cells (``primordial_cells``):
  * nH ~ logU(nH_lo, nH_hi) cm^-3, T ~ logU(T_lo, T_hi) K;
  * He mass fraction Y = 0.24: n_He = Y / (4 (1 - Y)) nH;
  * ionised fraction n(H+) = 1e-4 nH; n(H2) = 1e-6 nH;
    n(H-) = n(H2+) = n(He++) = n(He+) = 1e-12 nH; neutral H and He take the
    remainder of their nuclei;
  * electrons from charge neutrality;
  * ge [erg/g] from T through the solver's own T(ge) relation
    (gamma = 5/3 for every species), so the first temperature evaluation
    returns T;
  * stored as the reference's mass densities rho_s = n_s w_s 1.67e-24 g/cm^3
    (``input_is_number = False``), cells x species, species in state order;
  * dtf = 0.1 t_ff with t_ff = sqrt(3 pi / (32 G rho)).
  An optional unstable band puts a fraction of the cells at
  T ~ logU(1e4, 1e5) K with nH ~ logU(1e3, nH_hi).
"""

import numpy as np

KB = 1.3806504e-16
MH = 1.67e-24
G_NEWTON = 6.674e-8
GAMMA = 5.0 / 3.0

PRIMORDIAL_ORDER = ("H2_1", "H2_2", "H_1", "H_2", "H_m0", "He_1", "He_2", "He_3",
                    "de", "ge")
PRIMORDIAL_WEIGHTS = dict(H2_1=2.0, H2_2=2.0, H_1=1.00794, H_2=1.00794,
                          H_m0=1.00794, He_1=4.002602, He_2=4.002602,
                          He_3=4.002602, de=1.0)

# Named configurations: (nH range, T range, unstable fraction).
PRIMORDIAL_CONFIGS = {
    "config1": dict(nH=(1.0, 1e6), T=(10.0, 1e8), unstable=0.0, seed=20241),
    "config2": dict(nH=(1.0, 1e6), T=(10.0, 1e8), unstable=0.0, seed=20242),
    "config3": dict(nH=(1e-3, 1e12), T=(10.0, 0.999e9), unstable=0.05, seed=20243),
    # neutral gas only (T <= 1e4 K): every cell converges in a few hundred
    # sweeps; used to measure the solver's throughput without the stiff tail
    "cold": dict(nH=(1.0, 1e6), T=(10.0, 1e4), unstable=0.0, seed=20244),
    # ionised gas only (T >= 3e5 K): the stiff cells that run to the substep
    # cap; used to profile the per-cell critical path
    "hot": dict(nH=(1.0, 1e6), T=(3e5, 1e8), unstable=0.0, seed=20245),
    # the top decade of the tables (T up to just below the last bin, whose
    # upper neighbour the reference reads past the table's end)
    "top": dict(nH=(1e-3, 1e12), T=(1e8, 0.999e9), unstable=0.0, seed=20247),
}


def _logu(rng, lo, hi, n):
    return np.exp(rng.uniform(np.log(lo), np.log(hi), n))


def primordial_cells(ncells, config="config1", seed=None, dt_factor=0.1):
    """Return ``(state, dtf)``: state is (ncells, 10) float64 mass densities +
    ge in state order, dtf is (ncells,) float64 seconds."""
    cfg = PRIMORDIAL_CONFIGS[config]
    rng = np.random.Generator(np.random.PCG64(cfg["seed"] if seed is None else seed))
    nH = _logu(rng, *cfg["nH"], ncells)
    T = _logu(rng, *cfg["T"], ncells)
    if cfg["unstable"] > 0:
        band = rng.uniform(size=ncells) < cfg["unstable"]
        nb = int(band.sum())
        T[band] = _logu(rng, 1e4, 1e5, nb)
        nH[band] = _logu(rng, 1e3, cfg["nH"][1], nb)
    Y = 0.24
    nHe = Y / (4.0 * (1.0 - Y)) * nH
    n = {}
    n["H_2"] = 1e-4 * nH
    n["H2_1"] = 1e-6 * nH
    n["H_m0"] = 1e-12 * nH
    n["H2_2"] = 1e-12 * nH
    n["H_1"] = nH - n["H_2"] - n["H_m0"] - 2 * n["H2_1"] - 2 * n["H2_2"]
    n["He_3"] = 1e-12 * nH
    n["He_2"] = 1e-12 * nH
    n["He_1"] = nHe - n["He_2"] - n["He_3"]
    n["de"] = n["H_2"] - n["H_m0"] + n["H2_2"] + n["He_2"] + 2 * n["He_3"]
    density = sum(PRIMORDIAL_WEIGHTS[s] * n[s] for s in PRIMORDIAL_ORDER
                  if s not in ("de", "ge"))
    gsum = sum(n[s] / (GAMMA - 1.0) for s in PRIMORDIAL_ORDER if s != "ge")
    ge = T * KB * gsum / (density * MH)
    state = np.empty((ncells, len(PRIMORDIAL_ORDER)))
    for i, s in enumerate(PRIMORDIAL_ORDER):
        state[:, i] = ge if s == "ge" else n[s] * PRIMORDIAL_WEIGHTS[s] * MH
    rho = state[:, :-1].sum(axis=1)
    tff = np.sqrt(3.0 * np.pi / (32.0 * G_NEWTON * rho))
    return state, dt_factor * tff


# Oxygen ion-by-ion cells: H, He, O ions, electrons, energy (16 equations).
OXYGEN_ORDER = ("H_1", "H_2", "He_1", "He_2", "He_3", "O_1", "O_2", "O_3", "O_4", "O_5",
                "O_6", "O_7", "O_8", "O_9", "de", "ge")
OXYGEN_WEIGHTS = dict(H=1.00794, He=4.002602, O=15.9994)


def oxygen_cells(ncells, seed=20246, dt_range=(1e10, 1e12)):
    """Return ``(state, dtf)`` for the oxygen network (config 4).

    nH ~ logU(1e-4, 1e2) cm^-3, T ~ logU(1e4, 1e9) K, n_He = Y/(4(1-Y)) nH with
    Y = 0.24, n_O = 4.9e-4 nH; the ionisation state of each element is a
    seeded Dirichlet(1) draw over its stages; electrons from charge
    neutrality; ge from T with gamma = 5/3; dtf ~ logU(dt_range) s."""
    rng = np.random.Generator(np.random.PCG64(seed))
    nH = _logu(rng, 1e-4, 1e2, ncells)
    T = _logu(rng, 1e4, 1e9, ncells)
    n = {}
    for atom, nnuc, stages in (("H", nH, 2), ("He", 0.24 / (4 * 0.76) * nH, 3),
                               ("O", 4.9e-4 * nH, 9)):
        frac = rng.dirichlet(np.ones(stages), ncells)
        frac = np.maximum(frac, 1e-12)
        frac /= frac.sum(axis=1, keepdims=True)
        for i in range(stages):
            n["%s_%d" % (atom, i + 1)] = nnuc * frac[:, i]
    n["de"] = sum(n["%s_%d" % (a, i + 1)] * i for a, st in (("H", 2), ("He", 3), ("O", 9))
                  for i in range(st))
    w = {s: OXYGEN_WEIGHTS[s.split("_")[0]] for s in OXYGEN_ORDER if s not in ("de", "ge")}
    w["de"] = 1.0
    density = sum(w[s] * n[s] for s in OXYGEN_ORDER if s not in ("de", "ge"))
    gsum = sum(n[s] / (GAMMA - 1.0) for s in OXYGEN_ORDER if s != "ge")
    ge = T * KB * gsum / (density * MH)
    state = np.empty((ncells, len(OXYGEN_ORDER)))
    for i, s in enumerate(OXYGEN_ORDER):
        state[:, i] = ge if s == "ge" else n[s] * w[s] * MH
    return state, _logu(rng, *dt_range, ncells)
