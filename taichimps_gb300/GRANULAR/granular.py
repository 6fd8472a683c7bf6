"""
pair_style granular: composed normal / damping / tangential sub-models.

Mirrors taichimps ``PairGranular`` (src/taichimps/GRANULAR/granular.py:106-452):
the same sub-model names and ids, the same pair_coeff coefficient ordering, and
the same derived stiffnesses and damping constants (granular.py:94-103,
:207-269).  Unsupported sub-models raise at construction.
"""

from __future__ import annotations

import math
from typing import Any

from .base import GranularPair

NORMAL_HOOKE, NORMAL_HERTZ, NORMAL_HERTZ_MATERIAL = 0, 1, 2
DAMPING_NONE, DAMPING_VELOCITY, DAMPING_MASS_VELOCITY = 0, 1, 2
DAMPING_VISCOELASTIC, DAMPING_TSUJI, DAMPING_COEFF_RESTITUTION = 3, 4, 5
TANGENTIAL_NONE, TANGENTIAL_LINEAR_NOHISTORY, TANGENTIAL_LINEAR_HISTORY, TANGENTIAL_MINDLIN = 0, 1, 2, 3

_NORMAL = {"hooke": NORMAL_HOOKE, "hertz": NORMAL_HERTZ, "hertz/material": NORMAL_HERTZ_MATERIAL}
_DAMPING = {"none": DAMPING_NONE, "velocity": DAMPING_VELOCITY, "mass_velocity": DAMPING_MASS_VELOCITY,
            "viscoelastic": DAMPING_VISCOELASTIC, "tsuji": DAMPING_TSUJI,
            "coeff_restitution": DAMPING_COEFF_RESTITUTION}
_TANGENTIAL = {"none": TANGENTIAL_NONE, "linear_nohistory": TANGENTIAL_LINEAR_NOHISTORY,
               "linear_history": TANGENTIAL_LINEAR_HISTORY, "mindlin": TANGENTIAL_MINDLIN}

EPSILON = 1e-10
# LAMMPS gran_sub_mod_damping.cpp constants
TWOROOTFIVEBYSIX = 1.82574185835055380345   # 2 sqrt(5/6)
ROOTTHREEBYTWO = 1.22474487139158894067     # sqrt(3/2)


def mix_stiffness_e(e1: float, e2: float, poiss1: float, poiss2: float) -> float:
    """Effective Young's modulus of two materials (GranSubMod::mix_stiffnessE)."""
    return 1.0 / ((1 - poiss1 * poiss1) / e1 + (1 - poiss2 * poiss2) / e2)


def mix_stiffness_g(e1: float, e2: float, poiss1: float, poiss2: float) -> float:
    """Effective shear modulus of two materials (GranSubMod::mix_stiffnessG)."""
    return 1.0 / (2 * (2 - poiss1) * (1 + poiss1) / e1 + 2 * (2 - poiss2) * (1 + poiss2) / e2)


class PairGranular(GranularPair):
    def __init__(self, domain, normal: str, normal_coeffs, tangential: str = "none",
                 tangential_coeffs=None, damping: str = "viscoelastic", limit_damping: bool = False,
                 float_type: Any = None, rolling: str = "none", rolling_coeffs=None) -> None:
        super().__init__(domain, float_type=float_type)
        for kind, name, table in (("normal", normal, _NORMAL), ("damping", damping, _DAMPING),
                                  ("tangential", tangential, _TANGENTIAL)):
            if name not in table:
                raise ValueError(f"Unsupported pair granular {kind} model {name!r}; "
                                 f"implemented: {sorted(table)}")
        self.normal_id = _NORMAL[normal]
        self.damping_id = _DAMPING[damping]
        self.tangential_id = _TANGENTIAL[tangential]
        self.limit_damping = 1 if limit_damping else 0
        self.emod = 0.0
        self.poiss = 0.0
        if self.normal_id == NORMAL_HERTZ_MATERIAL:
            if len(normal_coeffs) != 3:
                raise ValueError("normal hertz/material takes E, damp, poisson")
            self.emod, cor, self.poiss = (float(c) for c in normal_coeffs)
            self.kn = (4.0 / 3.0) * mix_stiffness_e(self.emod, self.emod, self.poiss, self.poiss)
        else:
            if len(normal_coeffs) != 2:
                raise ValueError(f"normal {normal} takes k, damp")
            self.kn, cor = (float(c) for c in normal_coeffs)
        self.normal_damp = float(cor)
        self.damp = self._damping_coefficient(normal)
        self.normal_uses_contact_radius = self.normal_id != NORMAL_HOOKE
        self.kt = 0.0
        self.xt = 0.0
        self.mu = 0.0
        self.tangential_scales_k = self.tangential_id == TANGENTIAL_MINDLIN
        self.uses_history = self.tangential_id in (TANGENTIAL_LINEAR_HISTORY, TANGENTIAL_MINDLIN)
        if self.tangential_id != TANGENTIAL_NONE:
            self._setup_tangential(tangential, list(tangential_coeffs or []))
        # rolling resistance, RollingResistance (GRANULAR/rolling.py:16-50): k_roll, gamma_roll, mu_roll.
        # The reference defines the model but never calls it from a pair style; here it is wired into
        # pair granular as rolling.py writes it (see contact_law).
        if rolling not in ("none", "sds", "epsd"):
            raise ValueError(f"Unsupported pair granular rolling model {rolling!r}; implemented: "
                             "['epsd', 'none', 'sds']")
        self.rolling_id = 0 if rolling == "none" else 1
        self.k_roll = self.gamma_roll = self.mu_roll = 0.0
        if self.rolling_id:
            rc = list(rolling_coeffs or [])
            if len(rc) != 3:
                raise ValueError("rolling takes k_roll, gamma_roll, mu_roll")
            self.k_roll, self.gamma_roll, self.mu_roll = (float(c) for c in rc)
            self.uses_history = True
        self.submodels = {
            "normal": (normal, [float(c) for c in normal_coeffs]),
            "damping": (damping, []),
            "tangential": (tangential, [-1.0 if c is None else float(c) for c in (tangential_coeffs or [])]),
            "rolling": (rolling, [float(c) for c in (rolling_coeffs or [])] if self.rolling_id else []),
            "twisting": ("none", []), "heat": ("none", []),
        }
        p = self.params
        p.style = 4
        p.normal_id, p.damping_id, p.tangential_id = self.normal_id, self.damping_id, self.tangential_id
        p.limit_damping = self.limit_damping
        p.kn, p.kt, p.damp, p.xt, p.mu = self.kn, self.kt, self.damp, self.xt, self.mu
        p.rolling_id, p.k_roll, p.gamma_roll, p.mu_roll = self.rolling_id, self.k_roll, self.gamma_roll, self.mu_roll

    def _damping_coefficient(self, normal: str) -> float:
        """The damping sub-model's constant (granular.py:207-238)."""
        if self.damping_id in (DAMPING_TSUJI, DAMPING_COEFF_RESTITUTION):
            cor = self.normal_damp
            if not 0.0 < cor <= 1.0:
                raise ValueError("damping tsuji/coeff_restitution needs the normal model's damp "
                                 f"coefficient to be a restitution coefficient in (0, 1]; got {cor}")
            logcor = math.log(cor)
            if self.damping_id == DAMPING_TSUJI:
                # Marshall 2009 eq. 53 polynomial in e, times sqrt(2) for meff
                poly = (1.2728 - 4.2783 * cor + 11.087 * cor ** 2 - 22.348 * cor ** 3
                        + 27.467 * cor ** 4 - 18.022 * cor ** 5 + 4.8218 * cor ** 6)
                return poly * math.sqrt(2.0)
            if normal == "hooke":
                return -2 * logcor / math.sqrt(math.pi ** 2 + logcor ** 2)
            return -ROOTTHREEBYTWO * TWOROOTFIVEBYSIX * logcor / math.sqrt(math.pi ** 2 + logcor ** 2)
        return self.normal_damp

    def _setup_tangential(self, tangential: str, coeffs) -> None:
        if self.tangential_id == TANGENTIAL_LINEAR_NOHISTORY:
            if len(coeffs) != 2 or any(c is None for c in coeffs):
                raise ValueError("tangential linear_nohistory takes xt, mu")
            self.xt, self.mu = (float(c) for c in coeffs)
            return
        if len(coeffs) != 3:
            raise ValueError(f"tangential {tangential} takes k (or NULL), xt, mu")
        k_raw, xt, mu = coeffs
        if xt is None or mu is None:
            raise ValueError(f"tangential {tangential}: xt and mu cannot be NULL")
        self.xt, self.mu = float(xt), float(mu)
        if k_raw is None:
            if self.normal_id != NORMAL_HERTZ_MATERIAL:
                raise ValueError("a NULL tangential stiffness requires normal hertz/material, "
                                 "which is where E and Poisson's ratio come from")
            if self.tangential_id != TANGENTIAL_MINDLIN:
                raise ValueError("tangential linear_history needs an explicit stiffness")
            self.kt = 8.0 * mix_stiffness_g(self.emod, self.emod, self.poiss, self.poiss)
        else:
            self.kt = float(k_raw)
